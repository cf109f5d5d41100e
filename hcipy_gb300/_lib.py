"""ctypes binding of the C ABI in ``include/hcipy_gb300.h``.

The shared library is built in-tree (``hcipy_gb300/lib/libhcipy_gb300.so``).
There is no CPU path: every operator of this package calls into it, and
loading fails loudly when it has not been built or no CUDA device is present.
"""
import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'lib', 'libhcipy_gb300.so')

HX_OK = 0
HX_ERR_INVALID = -1
HX_ERR_CUDA = -2
HX_ERR_UNSUPPORTED = -3
HX_ERR_TIMEOUT = -4
HX_ERR_ALLOC = -5
HX_ERR_INJECTED = -6

HX_C64 = 0
HX_C128 = 1
HX_F32 = 2
HX_F64 = 3
HX_FORWARD = 0
HX_BACKWARD = 1
HX_ADJOINT = 2
HX_PREC_FP32 = 0
HX_PREC_SPLIT = 1
HX_SCHEDULE_LATENCY = 0
HX_SCHEDULE_THROUGHPUT = 1
HX_EPI_NONE = 0
HX_EPI_MUL = 1
HX_EPI_BABINET = 2
HX_TRACE_SPLIT_GEMM = 0
HX_TRACE_SIMT_GEMM = 1
HX_TRACE_FFT = 2
HX_TRACE_ATMOSPHERE = 3
HX_TRACE_DM = 4

c_int = ctypes.c_int
c_double = ctypes.c_double
c_size_t = ctypes.c_size_t
c_void_p = ctypes.c_void_p
c_ll = ctypes.c_longlong
P = ctypes.POINTER

# name -> (restype, argtypes); mirrors include/hcipy_gb300.h.
SIGNATURES = {
    'hx_last_error': (ctypes.c_char_p, []),
    'hx_version': (c_int, []),
    'hx_launch_count': (c_ll, []),
    'hx_trace_enable': (c_int, [c_int]),
    'hx_autotune': (c_int, [c_int]),
    'hx_autotune_entries': (c_int, []),
    'hx_autotune_entry': (c_int, [c_int, P(c_ll), P(c_int), P(c_int), P(c_int), P(ctypes.c_float)]),
    'hx_autotune_clear': (c_int, []),
    'hx_efc_step': (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_double, c_void_p,
                            c_void_p]),
    'hx_intensity_sums_workspace_bytes': (c_size_t, [c_ll, c_int]),
    'hx_intensity_sums': (c_int, [c_void_p, c_int, c_ll, c_int, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    'hx_intensity_sums_grad': (c_int, [c_void_p, c_int, c_ll, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    'hx_influence_apply': (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p,
                                   c_void_p]),
    'hx_influence_apply_transpose': (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p,
                                             c_void_p, c_void_p]),
    'hx_influence_apply_transpose_blocked': (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int,
                                                     c_void_p, c_void_p, c_void_p]),
    'hx_phase_apply': (c_int, [c_ll, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_double, c_void_p, c_void_p]),
    'hx_phase_apply_grad': (c_int, [c_ll, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_double, c_void_p,
                                    c_void_p, c_void_p, c_void_p]),
    'hx_atmosphere_extrude': (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p,
                                      c_void_p, c_int, c_void_p, c_int, c_void_p]),
    'hx_atmosphere_extrude_layers': (c_int, [c_void_p, c_int, c_int, c_void_p]),
    'hx_atmosphere_shift': (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, P(c_double), P(c_double),
                                    c_void_p, c_int, c_void_p]),
    'hx_atmosphere_shift_layers': (c_int, [P(c_void_p), c_int, c_int, c_int, c_int, c_int, P(c_int), P(c_int),
                                           P(c_double), P(c_double), P(c_void_p), c_void_p, c_int, c_void_p]),
    'hx_mft_plan_set_schedule': (c_int, [c_void_p, c_int]),
    'hx_atmosphere_combine': (c_int, [P(c_void_p), c_int, c_ll, c_void_p, c_int, c_void_p]),
    'hx_trace_read': (c_int, [c_int, P(c_ll), P(c_double), P(c_double), c_int]),
    'hx_mft_plan_create': (c_int, [c_int, c_int, c_int, c_int, P(c_double), P(c_double), P(c_double), P(c_double),
                                   P(c_double), P(c_double), P(c_double), P(c_double), c_int, c_int, c_void_p,
                                   P(c_void_p)]),
    'hx_mft_workspace_bytes': (c_size_t, [c_void_p, c_int, c_int]),
    'hx_mft_execute': (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_double, c_double, c_void_p, c_size_t,
                               c_void_p]),
    'hx_mft_execute_ex': (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_double, c_double, c_int, c_void_p,
                                  c_void_p, c_void_p, c_size_t, c_void_p]),
    'hx_mft_plan_destroy': (c_int, [c_void_p]),
    'hx_mft_plan_status': (c_int, [c_void_p, c_int]),
    'hx_mft_execute_io': (c_int, [c_void_p, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_double, c_double, c_int,
                                  c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    'hx_lyot_workspace_bytes': (c_size_t, [c_void_p, c_void_p, c_int]),
    'hx_mft_execute_phase': (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_double, c_void_p, c_int, c_double,
                                     c_double, c_void_p, c_size_t, c_void_p]),
    'hx_lyot_execute': (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_double, c_double,
                                c_double, c_double, c_double, c_double, c_void_p, c_int, c_void_p, c_int, c_void_p,
                                c_size_t, c_void_p]),
    'hx_mft_execute_noalloc': (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_double, c_double, c_void_p]),
    'hx_fft_plan_create': (c_int, [c_int, P(c_int), P(c_int), P(c_int), P(c_int), P(c_int), P(P(c_double)),
                                   P(P(c_double)), c_double, c_double, c_int, c_void_p, P(c_void_p)]),
    'hx_fft_workspace_bytes': (c_size_t, [c_void_p, c_int, c_int]),
    'hx_fft_execute': (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    'hx_fft_plan_destroy': (c_int, [c_void_p]),
    'hx_filter_plan_create': (c_int, [c_int, P(c_int), P(c_int), P(c_int), c_void_p, c_int, c_void_p, P(c_void_p)]),
    'hx_filter_workspace_bytes': (c_size_t, [c_void_p, c_int]),
    'hx_filter_execute': (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    'hx_filter_plan_destroy': (c_int, [c_void_p]),
    'hx_czt_plan_create': (c_int, [c_int, c_int, c_double, c_double, c_double, c_double, P(c_double), P(c_double),
                                   c_int, c_void_p, P(c_void_p)]),
    'hx_czt_execute': (c_int, [c_void_p, c_int, c_int, c_void_p, c_ll, c_ll, c_ll, c_void_p, c_ll, c_ll, c_ll,
                               c_void_p]),
    'hx_czt_plan_destroy': (c_int, [c_void_p]),
    'hx_fresnel_transfer_function': (c_int, [c_int, c_int, c_double, c_double, c_double, c_double, c_double,
                                             c_double, c_int, c_int, c_void_p, c_void_p]),
    'hx_fresnel_impulse_response': (c_int, [c_int, c_int, c_double, c_double, c_double, c_double, c_double,
                                            c_double, c_double, c_int, c_int, c_void_p, c_void_p]),
    'hx_asp_transfer_function': (c_int, [c_int, c_int, c_double, c_double, c_double, c_double, c_double, c_double,
                                         c_int, c_int, c_void_p, c_void_p]),
    'hx_asp_impulse_response': (c_int, [c_int, c_int, c_double, c_double, c_double, c_double, c_double, c_double,
                                        c_int, c_int, c_void_p, c_void_p]),
}

_lib = None


class Extrusion(ctypes.Structure):
    """``hx_extrusion``: one extrusion step of one layer (device pointers, ring sizes and offsets)."""
    _fields_ = [('ring', c_void_p), ('stencil_idx', c_void_p), ('A', c_void_p), ('B', c_void_p),
                ('noise', c_void_p), ('ny', c_int), ('nx', c_int), ('row0', c_int), ('col0', c_int),
                ('where', c_int), ('nst', c_int), ('nb', c_int)]


class HXError(RuntimeError):
    """A failure reported by the CUDA library (status code and message)."""

    def __init__(self, code, message):
        RuntimeError.__init__(self, '%s (status %d)' % (message, code))
        self.code = code


def load():
    """Load the shared library; raise ImportError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError('hcipy_gb300: the CUDA library %s is not built; run `python -m hcipy_gb300._build` '
                          '(or __graft_entry__.build()) first' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def lib():
    lib_ = load()
    if not torch.cuda.is_available():
        raise RuntimeError('hcipy_gb300 needs a CUDA device (GB300, sm_103a); no CPU path exists')
    return lib_


def check(rc, what=''):
    if rc == HX_OK:
        return
    msg = load().hx_last_error().decode(errors='replace')
    if what:
        msg = '%s: %s' % (what, msg)
    if rc == HX_ERR_INVALID:
        raise ValueError(msg)
    raise HXError(rc, msg)


def stream_handle(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def dptr(t):
    """Device address of a tensor's data.  A conjugate view (``t.conj()``) shares the memory of its base and only
    flags the conjugation, which a kernel cannot see: such views are refused (resolve them first)."""
    if t.is_complex() and t.is_conj():
        raise ValueError('a lazily conjugated tensor was passed to the library; call resolve_conj() first')
    return ctypes.c_void_p(t.data_ptr())


def darr(a):
    """A float64 host array as a ctypes pointer (None -> NULL); keeps the buffer alive via the return tuple."""
    import numpy as np
    if a is None:
        return None, None
    buf = np.ascontiguousarray(a, dtype=np.float64)
    return buf, buf.ctypes.data_as(P(c_double))


def iarr(values):
    """A host int array as a ctypes pointer; returns (buffer, pointer)."""
    buf = (ctypes.c_int * len(values))(*[int(v) for v in values])
    return buf, ctypes.cast(buf, P(c_int))


def carr(values):
    """A host complex array as interleaved float64 (buffer, pointer); None -> (None, None)."""
    import numpy as np
    if values is None:
        return None, None
    buf = np.ascontiguousarray(np.asarray(values, dtype=np.complex128)).view(np.float64)
    return buf, buf.ctypes.data_as(P(c_double))


def ptr_array(ptrs):
    """An array of double* (None -> NULL) for the per-axis factor arguments."""
    arr = (P(c_double) * len(ptrs))(*[p if p is not None else P(c_double)() for p in ptrs])
    return arr, ctypes.cast(arr, P(P(c_double)))


def workspace(nbytes, device):
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=device)


def dtype_code(dt):
    if dt == torch.complex64:
        return HX_C64
    if dt == torch.complex128:
        return HX_C128
    if dt == torch.float32:
        return HX_F32
    if dt == torch.float64:
        return HX_F64
    raise ValueError('unsupported dtype %s' % dt)


def launch_count():
    return int(load().hx_launch_count())


def autotune(on=True):
    """Measure the split-GEMM tile candidates of each new GEMM shape once and keep the fastest."""
    check(lib().hx_autotune(1 if on else 0), 'hx_autotune')


def autotune_entries():
    return int(lib().hx_autotune_entries())


def autotune_table():
    """[(shape (row tiles, columns, z, K steps), [(bn, ksplit, ms), ...] best first)] of the autotuner."""
    out = []
    for i in range(autotune_entries()):
        shape = (ctypes.c_longlong * 4)()
        n = ctypes.c_int()
        bn, ks = (ctypes.c_int * 8)(), (ctypes.c_int * 8)()
        ms = (ctypes.c_float * 8)()
        check(lib().hx_autotune_entry(i, shape, ctypes.byref(n), bn, ks, ms), 'hx_autotune_entry')
        cands = sorted([(bn[k], ks[k], round(float(ms[k]), 4)) for k in range(n.value)], key=lambda c: c[2])
        out.append((tuple(shape), cands))
    return out


def trace_enable(on=True):
    """Bracket every GEMM and FFT pass the library launches with CUDA events on its stream."""
    check(lib().hx_trace_enable(1 if on else 0), 'hx_trace_enable')


def trace_read(kind, reset=True):
    """(launches, device milliseconds, algorithmic work) of one kernel family since the last reset."""
    n = ctypes.c_longlong()
    ms = ctypes.c_double()
    work = ctypes.c_double()
    check(lib().hx_trace_read(kind, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(work), 1 if reset else 0),
          'hx_trace_read')
    return int(n.value), float(ms.value), float(work.value)
