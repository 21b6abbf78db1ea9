"""CPU oracle for the spinor-gpe split-step path.

TEST INFRASTRUCTURE ONLY.  This package restates, on the CPU, the algorithm
of the original spinor-gpe propagator so that the CUDA solver can be checked
against it.  Only the test suite, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import it, and only as the checker or the
timed CPU baseline -- never as a code path of the solver itself.

Parity status: pinned.  ``tests/test_oracle_golden.py`` checks this
restatement against golden vectors produced by running the original package
(``tests/golden/make_golden.py``) on the same inputs, in complex128 and in
complex64.
"""
from .split_step import (OracleInputs, OraclePropagator, calc_pops,  # noqa: F401
                         coupling_op, evolution_op, fft_2d, ifft_2d, norm,
                         fft_1d, ifft_1d, inputs_from_arrays)
