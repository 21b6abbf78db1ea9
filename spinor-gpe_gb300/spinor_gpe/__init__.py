"""GB300 split-step solver for the pseudospin-1/2 Gross-Pitaevskii equation,
with the Python interface of spinor-gpe (``spinor_gpe.pspinor.pspinor``,
``spinor_gpe.pspinor.tensor_propagator``, ``spinor_gpe.pspinor.tensor_tools``).

The time stepping runs in the native CUDA library ``libspinor_gb300.so``
(built by ``spinor-gpe_gb300/build_native.py``).
"""
