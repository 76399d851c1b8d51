"""Minimal stand-in for numba, used only when importing the reference to make golden vectors.

The reference imports ``numba.njit`` and ``numba.prange`` at module load (khepri/fourier.py:71);
the functions they decorate (``dft``, ``slow_dft``, ``idft2``) are not on the Crystal solve path.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


jit = njit
prange = range
