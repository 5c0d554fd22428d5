"""Stand-in for numba, used only to import the reference's galaxy_formation/sph.py in this
container (numba is not installed). `njit` returns the function unchanged and `prange` is
`range`, so the reference code runs as plain Python/NumPy with the same float64
arithmetic (without fastmath reassociation). TEST INFRASTRUCTURE ONLY."""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(f):
        return f

    return wrap


prange = range
