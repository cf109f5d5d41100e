"""array_api_compat stand-in for numpy-only use."""
import numpy as np


def array_namespace(*arrays, **kwargs):
    return np


def is_numpy_array(x):
    return isinstance(x, (np.ndarray, np.generic))


def _false(x):
    return False


is_cupy_array = is_jax_array = is_torch_array = is_dask_array = _false


def is_numpy_namespace(xp):
    return xp is np


is_cupy_namespace = is_jax_namespace = is_torch_namespace = is_array_api_strict_namespace = _false
