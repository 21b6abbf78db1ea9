"""File-name helper of spinor-gpe's ``plotting_tools``.

Only ``next_available_path`` (``spinor_gpe/pspinor/plotting_tools.py:13-37``)
is provided: the propagator names its sampled-wavefunction files with it.
The matplotlib plotting functions of the original are outside this package.
"""
import os


def next_available_path(file_name, trial_name, ext=''):
    """First ``<file_name><i>-<trial_name><ext>`` (i = 1, 2, ...) that does
    not exist yet."""
    i = 1
    test_path = f'{file_name}{i}-{trial_name}{ext}'
    while os.path.exists(test_path):
        i += 1
        test_path = f'{file_name}{i}-{trial_name}{ext}'
    return test_path
