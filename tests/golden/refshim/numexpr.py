"""numexpr stand-in: evaluates the expression with numpy in float64/complex128.

The reference calls numexpr.evaluate for exp/abs/real/imag element-wise work; the
numpy evaluation computes the same quantities.  Used only to import the
reference for fixture generation.
"""
import sys
import numpy as np

_NS = {'exp': np.exp, 'real': np.real, 'imag': np.imag, 'abs': np.abs,
       'sqrt': np.sqrt, 'sin': np.sin, 'cos': np.cos, 'log': np.log,
       'arctan2': np.arctan2, 'where': np.where, 'conj': np.conj}


def evaluate(expr, local_dict=None, global_dict=None, out=None, **kwargs):
    if local_dict is None:
        frame = sys._getframe(1)
        local_dict = dict(frame.f_globals)
        local_dict.update(frame.f_locals)
    env = dict(_NS)
    env.update({k: (np.asarray(v) if not np.isscalar(v) else v) for k, v in local_dict.items()})
    res = eval(expr, {'__builtins__': {}}, env)
    if out is not None:
        out[...] = res
        return out
    return np.asarray(res)


def set_num_threads(n):
    return 1


def detect_number_of_cores():
    return 1
