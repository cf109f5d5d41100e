"""numba stand-in: identity decorators (the functions run as plain Python)."""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        f = args[0]
        f.py_func = f
        return f

    def deco(f):
        f.py_func = f
        return f
    return deco


jit = njit
prange = range
