"""Fourier operators behind HCIPy's operator API (hcipy/fourier/*), on the GPU.

``FourierTransform`` keeps the reference interface (hcipy/fourier/fourier_transform.py:17-183):
``input_grid``, ``output_grid``, ``forward(field)``, ``backward(field)``,
classmethods ``is_supported``, ``check_if_supported`` (raises ValueError) and
``compute_complexity``.  Tensor fields (leading dimensions) are transformed as
one batched launch, not a Python loop.  The output dtype follows the input bit
depth: complex64 in -> complex64 out, anything else -> complex128.
"""
import ctypes
import math
from collections.abc import Iterable
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .field import Field, CartesianGrid, RegularCoords, as_tensor, complex_dtype_for

# ---------------------------------------------------------------------------
# Base class and helpers
# ---------------------------------------------------------------------------


@dataclass(frozen=True)
class ComputationalComplexity:
    num_multiplications: int = 0
    num_additions: int = 0
    expected_execution_time: float = 0

    @property
    def num_operations(self):
        return self.num_multiplications + self.num_additions


class FourierTransform(object):
    """Base class of the Fourier operators (hcipy/fourier/fourier_transform.py:17-183)."""

    def forward(self, field):
        raise NotImplementedError()

    def backward(self, field):
        raise NotImplementedError()

    @classmethod
    def is_supported(cls, input_grid, output_grid):
        try:
            cls.check_if_supported(input_grid, output_grid)
        except ValueError:
            return False
        return True

    @classmethod
    def check_if_supported(cls, input_grid, output_grid):
        raise NotImplementedError()

    @classmethod
    def compute_complexity(cls, input_grid, output_grid):
        raise NotImplementedError()


def _is_cartesian(grid):
    try:
        return bool(grid.is_('cartesian'))
    except Exception:
        return False


def _prepare_input(field, grid):
    """Device tensor of a field, cast to the complex dtype of its bit depth and made contiguous."""
    t = as_tensor(field)
    cdt = complex_dtype_for(t.dtype)
    if t.dtype != cdt:
        t = t.to(cdt)
    t = t.contiguous()
    if t.shape[-1] != grid.size:
        raise ValueError('The field has %d points per component, the grid %d.' % (t.shape[-1], grid.size))
    return t


def _axis_weights(grid):
    """Per-axis weights of a separated grid, or None when its weight is one scalar (regular grids)."""
    if getattr(grid, 'is_regular', False):
        return None
    axes = []
    for x in grid.separated_coords:
        x = np.asarray(x, np.float64)
        if len(x) > 1:
            axes.append(np.concatenate(([x[1] - x[0]], (x[2:] - x[:-2]) / 2, [x[-1] - x[-2]])))
        else:
            axes.append(np.ones(1))
    return axes


def _broadcast_mask(mask, grid, dtype):
    """One complex field of ``grid`` (a scalar, Field, tensor or array) as a contiguous device tensor."""
    if np.isscalar(mask):
        return torch.full((grid.size,), complex(mask), dtype=dtype, device='cuda')
    m = as_tensor(mask).to(dtype)
    if m.numel() == 1:
        m = m.reshape(1).expand(grid.size)
    if m.shape[-1] != grid.size or m.numel() != grid.size:
        raise ValueError('A fused mask must be one field of the destination grid.')
    return m.reshape(grid.size).contiguous().resolve_conj()


def _scalar_weight(grid):
    return float(np.prod(np.asarray(grid.delta, np.float64)))


# ---------------------------------------------------------------------------
# Matrix Fourier transform
# ---------------------------------------------------------------------------

PRECISIONS = {'fp32': _lib.HX_PREC_FP32, 'split': _lib.HX_PREC_SPLIT}
SCHEDULES = {'latency': _lib.HX_SCHEDULE_LATENCY, 'throughput': _lib.HX_SCHEDULE_THROUGHPUT}


class _MftPlan(object):
    """Owner of one C plan (phase matrices of one dtype and precision)."""

    def __init__(self, x, y, u, v, win, wout, dtype_code, precision_code):
        lib = _lib.lib()
        keep = []
        ptrs = []
        for arr in (x, y, u, v):
            buf, p = _lib.darr(arr)
            keep.append(buf)
            ptrs.append(p)
        wptrs = []
        for arr in (win[0] if win else None, win[1] if win else None, wout[0] if wout else None,
                    wout[1] if wout else None):
            buf, p = _lib.darr(arr)
            keep.append(buf)
            wptrs.append(p)
        handle = ctypes.c_void_p()
        rc = lib.hx_mft_plan_create(len(x), len(y), len(u), len(v), *ptrs, *wptrs, dtype_code, precision_code,
                                    _lib.stream_handle(), ctypes.byref(handle))
        _lib.check(rc, 'hx_mft_plan_create')
        self.handle = handle
        self.lib = lib
        self.dtype_code = dtype_code

    def workspace_bytes(self, direction, batch):
        return int(self.lib.hx_mft_workspace_bytes(self.handle, direction, batch))

    def execute(self, direction, batch, inp, out, alpha, workspace=None, epilogue=_lib.HX_EPI_NONE, mask=None,
                src=None):
        nbytes = self.workspace_bytes(direction, batch)
        if workspace is None or workspace.numel() < nbytes:
            workspace = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=inp.device)
        rc = self.lib.hx_mft_execute_ex(self.handle, direction, batch, _lib.dptr(inp), _lib.dptr(out),
                                        float(alpha.real), float(alpha.imag), epilogue,
                                        None if mask is None else _lib.dptr(mask),
                                        None if src is None else _lib.dptr(src),
                                        _lib.dptr(workspace), nbytes, _lib.stream_handle())
        _lib.check(rc, 'hx_mft_execute_ex')

    def execute_io(self, direction, batch, inp, out, alpha, epilogue=_lib.HX_EPI_NONE, mask=None, src=None):
        """Split plans: complex64 or complex128 input, output and Babinet source (dtype taken from the tensors)."""
        nbytes = self.workspace_bytes(direction, batch)
        workspace = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=inp.device)
        rc = self.lib.hx_mft_execute_io(self.handle, direction, batch, _lib.dptr(inp), _lib.dtype_code(inp.dtype),
                                        _lib.dptr(out), _lib.dtype_code(out.dtype), float(alpha.real),
                                        float(alpha.imag), epilogue, None if mask is None else _lib.dptr(mask),
                                        None if src is None else _lib.dptr(src),
                                        _lib.dtype_code(src.dtype) if src is not None else _lib.HX_C64,
                                        _lib.dptr(workspace), nbytes, _lib.stream_handle())
        _lib.check(rc, 'hx_mft_execute_io')

    def execute_phase(self, batch, inp, screen, scale, out, alpha):
        """Split plans, forward: complex64 fields times exp(i scale screen), the phase applied while slicing."""
        nbytes = self.workspace_bytes(_lib.HX_FORWARD, batch)
        workspace = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=inp.device)
        rc = self.lib.hx_mft_execute_phase(self.handle, batch, _lib.dptr(inp), _lib.dptr(screen), float(scale),
                                           _lib.dptr(out), _lib.dtype_code(out.dtype), float(alpha.real),
                                           float(alpha.imag), _lib.dptr(workspace), nbytes, _lib.stream_handle())
        _lib.check(rc, 'hx_mft_execute_phase')

    def set_schedule(self, code):
        _lib.check(self.lib.hx_mft_plan_set_schedule(self.handle, code), 'hx_mft_plan_set_schedule')

    def status(self, reset=True):
        """Status of the plan's bounded device waits (0 = fine); synchronizes with the device."""
        return int(self.lib.hx_mft_plan_status(self.handle, 1 if reset else 0))

    def __del__(self):
        try:
            if self.handle:
                self.lib.hx_mft_plan_destroy(self.handle)
        except Exception:
            pass


class MatrixFourierTransform(FourierTransform):
    """Matrix Fourier transform (hcipy/fourier/matrix_fourier_transform.py:8-310) as two device GEMMs.

    ``precision`` selects the GEMM arithmetic: ``'fp32'`` (default) is the plain
    drop-in (complex64 fields on FP32 CUDA cores, complex128 fields in FP64);
    ``'split'`` runs on tcgen05 tensor cores with fixed-point fp16 slices and
    exact sums (~29-bit operands), takes complex64 or complex128 fields and
    returns complex128, since its results hold more than a complex64 can.  ``precompute_matrices`` and
    ``allocate_intermediate`` are accepted for API compatibility: the phase
    matrices are always kept on the device and the intermediate is scratch from
    torch's caching allocator.  ``schedule`` ('latency', default, or 'throughput') is the
    tile policy of the GEMMs: 'latency' narrows tiles (CUDA cores) or splits K (tensor
    cores) until a small transform occupies the GPU; 'throughput' is for transforms that
    run beside others (several streams, parallel graph branches), see
    ``hx_mft_plan_set_schedule``.
    """

    def __init__(self, input_grid, output_grid, precompute_matrices=None, allocate_intermediate=None,
                 precision='fp32', schedule='latency'):
        self.check_if_supported(input_grid, output_grid)
        self.input_grid = input_grid
        self.output_grid = output_grid
        self.ndim = input_grid.ndim
        self.shape_input = tuple(int(d) for d in np.asarray(input_grid.dims)[::-1])
        self.shape_output = tuple(int(d) for d in np.asarray(output_grid.dims)[::-1])
        self.precompute_matrices = True if precompute_matrices is None else precompute_matrices
        self.allocate_intermediate = True if allocate_intermediate is None else allocate_intermediate
        if precision not in PRECISIONS:
            raise ValueError('precision must be one of %s' % sorted(PRECISIONS))
        self.precision = precision
        if schedule not in SCHEDULES:
            raise ValueError('schedule must be one of %s' % sorted(SCHEDULES))
        self._schedule = schedule

        xs = [np.asarray(c, np.float64) for c in input_grid.separated_coords]
        us = [np.asarray(c, np.float64) for c in output_grid.separated_coords]
        if self.ndim == 1:
            self._coords = (xs[0], np.zeros(1), us[0], np.zeros(1))
        else:
            self._coords = (xs[0], xs[1], us[0], us[1])
        win = _axis_weights(input_grid)
        wout = _axis_weights(output_grid)
        if self.ndim == 1:
            win = None if win is None else (win[0], np.ones(1))
            wout = None if wout is None else (wout[0], np.ones(1))
        self._win = win
        self._wout = wout
        self._w_in_scalar = 1.0 if win is not None else _scalar_weight(input_grid)
        self._w_out_scalar = 1.0 if wout is not None else _scalar_weight(output_grid)
        self._plans = {}

    # -- plans ---------------------------------------------------------------
    def _plan(self, cdt):
        code = _lib.HX_C64 if cdt == torch.complex64 else _lib.HX_C128
        prec = PRECISIONS[self.precision]
        if prec == _lib.HX_PREC_SPLIT:
            code = _lib.HX_C64  # split plans take either field dtype
        key = (code, prec)
        plan = self._plans.get(key)
        if plan is None:
            plan = _MftPlan(*self._coords, self._win, self._wout, code, prec)
            plan.set_schedule(SCHEDULES[self._schedule])
            self._plans[key] = plan
        return plan

    @property
    def schedule(self):
        return self._schedule

    @schedule.setter
    def schedule(self, schedule):
        if schedule not in SCHEDULES:
            raise ValueError('schedule must be one of %s' % sorted(SCHEDULES))
        self._schedule = schedule
        for plan in self._plans.values():
            plan.set_schedule(SCHEDULES[schedule])

    def _run(self, field, src_grid, dst_grid, direction, alpha, epilogue=_lib.HX_EPI_NONE, mask=None, src=None,
             out=None):
        t = _prepare_input(field, src_grid)
        batch_shape = tuple(t.shape[:-1])
        batch = int(np.prod(batch_shape)) if batch_shape else 1
        split = self.precision == 'split'
        if out is None:
            out_dtype = torch.complex128 if split else t.dtype
            out = torch.empty(batch_shape + (dst_grid.size,), dtype=out_dtype, device=t.device)
        if mask is not None:
            mask = _broadcast_mask(mask, dst_grid, torch.complex64 if split else t.dtype)
        if src is not None:
            src = src.contiguous() if split else src.to(t.dtype).contiguous()
            if tuple(src.shape) != tuple(out.shape):
                src = src.expand(out.shape).contiguous()
        if batch > 0:
            plan = self._plan(t.dtype)
            if self.precision == 'split':
                plan.execute_io(direction, batch, t, out, alpha, epilogue=epilogue, mask=mask, src=src)
            else:
                plan.execute(direction, batch, t, out, alpha, epilogue=epilogue, mask=mask, src=src)
        return Field(out, dst_grid)

    # -- operator API ----------------------------------------------------------
    def forward(self, field):
        """Forward MFT: w_in * M1 . E . M2 (matrix_fourier_transform.py:133-176)."""
        return self._run(field, self.input_grid, self.output_grid, _lib.HX_FORWARD, complex(self._w_in_scalar))

    def backward(self, field):
        """Inverse MFT: w_out/(2 pi)^d * M1^H . F . M2^H (matrix_fourier_transform.py:179-224)."""
        alpha = complex(self._w_out_scalar / (2 * np.pi)**self.ndim)
        return self._run(field, self.output_grid, self.input_grid, _lib.HX_BACKWARD, alpha)

    def adjoint(self, field):
        """Conjugate transpose of ``forward`` (w_in * M1^H . F . M2^H); not part of the reference API."""
        return self._run(field, self.output_grid, self.input_grid, _lib.HX_ADJOINT, complex(self._w_in_scalar))

    @classmethod
    def check_if_supported(cls, input_grid, output_grid):
        """matrix_fourier_transform.py:227-253."""
        if not input_grid.is_separated or not _is_cartesian(input_grid):
            raise ValueError('The input_grid must be separable in cartesian coordinates.')
        if not output_grid.is_separated or not _is_cartesian(output_grid):
            raise ValueError('The output_grid must be separable in cartesian coordinates.')
        if input_grid.ndim not in [1, 2]:
            raise ValueError('The input_grid must be one- or two-dimensional.')
        if input_grid.ndim != output_grid.ndim:
            raise ValueError('The input_grid must have the same dimensions as the output_grid.')

    @classmethod
    def compute_complexity(cls, input_grid, output_grid):
        """Operation count and predicted time as the reference planner computes them
        (matrix_fourier_transform.py:256-310), so ``planner='estimate'`` makes the reference's choice."""
        cls.check_if_supported(input_grid, output_grid)
        mults, adds = _mft_operation_count(input_grid, output_grid)
        return ComputationalComplexity(mults, adds, reference_seconds('mft', mults + adds))

    @classmethod
    def gpu_execution_time(cls, input_grid, output_grid):
        """GB300 time estimate: two complex GEMM launches at the CUDA-core rate."""
        cls.check_if_supported(input_grid, output_grid)
        if input_grid.ndim == 1:
            cmacs = input_grid.size * output_grid.size
        else:
            nx, ny = (int(d) for d in input_grid.dims)
            nu, nv = (int(d) for d in output_grid.dims)
            cmacs = ny * nx * nu + nv * ny * nu
        return cost_model.mft_seconds(8 * cmacs)


def _mft_operation_count(input_grid, output_grid):
    """Real multiplications and additions of the MFT as the reference counts them.

    The reference unpacks ``grid.shape`` (which is (Ny, Nx)) into names ordered
    (x, y), so its count uses Nx_in*Ny_in*Nx_out + Ny_in*Ny_out*Nx_out; that order
    is kept so that the planner's choices match.
    """
    if input_grid.ndim == 1:
        cmul = input_grid.size * output_grid.size
        cadd = (input_grid.size - 1) * output_grid.size
    else:
        ny_in, nx_in = (int(d) for d in np.asarray(input_grid.dims)[::-1])
        ny_out, nx_out = (int(d) for d in np.asarray(output_grid.dims)[::-1])
        a_in, b_in = ny_in, nx_in      # the reference's (N_in_x, N_in_y)
        a_out, b_out = ny_out, nx_out  # the reference's (N_out_x, N_out_y)
        cmul = b_in * a_in * b_out + a_in * a_out * b_out + input_grid.size
        cadd = b_out * a_in * (b_in - 1) + a_out * b_out * (a_in - 1)
    return 4 * cmul, 2 * cmul + 2 * cadd


# Execution-time model of the reference planner, t_ms = exp(a) * GFLOP^b + exp(c), with the
# coefficients of its default configuration (hcipy/config/default_config.yaml:10-44,
# fitted by the reference on its CPU; hcipy/fourier/fourier_transform.py:159-183).
REFERENCE_TIME_COEFFICIENTS = {
    'fft': (3.746, 0.881, -4.749),
    'mft': (1.667, 0.716, -4.624),
    'zfft': (4.093, 0.847, -2.973),
}


def reference_seconds(method, num_operations):
    a, b, c = REFERENCE_TIME_COEFFICIENTS[method]
    return (math.exp(a) * (num_operations / 1e9)**b + math.exp(c)) * 1e-3


# ---------------------------------------------------------------------------
# GB300 cost model of the planner
# ---------------------------------------------------------------------------


class _CostModel(object):
    """Predicted device time of each method; replaces the CPU-fitted coefficients of the reference
    planner (hcipy/fourier/fourier_transform.py:159-183, hcipy/config/default_config.yaml:10-44).

    ``t = launches * launch_s + max(bytes / hbm_bytes, flops / rate)``: the MFT is
    two complex GEMM launches at the FP32 CUDA-core rate measured on a GB300; a
    zero-padded FFT or a zoom FFT is one line-FFT launch per axis, bound by the
    HBM traffic of its source, intermediate and destination planes or by the
    shared-memory butterflies.
    """
    launch_s = 3e-6
    mft_flops = 30e12
    fft_flops = 15e12
    hbm_bytes = 5e12

    def mft_seconds(self, ops):
        return 2 * self.launch_s + ops / self.mft_flops

    def fft_seconds(self, n_internal, n_in, n_out, passes=2, n_mid=0, itemsize=8):
        traffic = (n_in + n_out + 2 * n_mid) * itemsize
        flops = 5.0 * n_internal * max(math.log2(max(n_internal, 2)), 1)
        return passes * self.launch_s + max(traffic / self.hbm_bytes, flops / self.fft_flops)


cost_model = _CostModel()


# ---------------------------------------------------------------------------
# FFT-grid algebra (hcipy/fourier/fast_fourier_transform.py:23-154)
# ---------------------------------------------------------------------------


def _as_tuple(v, n):
    if isinstance(v, Iterable) and not isinstance(v, str):
        v = tuple(v)
        return v * n if len(v) == 1 else v
    return (v,) * n


def make_fft_grid(input_grid, q=1, fov=1, shift=0):
    """The grid an FFT of ``input_grid`` produces (fast_fourier_transform.py:23-62)."""
    n = input_grid.ndim
    q = _as_tuple(q, n)
    fov = _as_tuple(fov, n)
    shift = _as_tuple(shift, n)
    if not input_grid.is_regular:
        raise ValueError('The input_grid must be regular.')
    if not _is_cartesian(input_grid):
        raise ValueError('The input_grid must be cartesian.')
    dims_in = [int(d) for d in input_grid.dims]
    delta_in = [float(d) for d in input_grid.delta]
    q = tuple(round(qi * d) / d for qi, d in zip(q, dims_in))
    delta = tuple(float((2 * math.pi / (d * s)) / qi) for d, s, qi in zip(delta_in, dims_in, q))
    dims = tuple(int(d * f * qi) for d, f, qi in zip(dims_in, fov, q))
    zero = tuple(float(di * (-dim / 2 + (dim % 2) * 0.5) + si) for di, dim, si in zip(delta, dims, shift))
    return CartesianGrid(RegularCoords(delta, dims, zero))


def get_fft_parameters(fft_grid, input_grid):
    """Recover (q, fov, shift) of an FFT grid, or raise ValueError (fast_fourier_transform.py:64-130)."""
    if not input_grid.is_regular:
        raise ValueError('The input grid must be regular to reconstruct an fft grid.')
    if not fft_grid.is_regular:
        raise ValueError('The fft grid is not regular and therefore cannot be an fft grid.')
    if input_grid.ndim != fft_grid.ndim:
        raise ValueError('The fft grid does not have the same number of dimensions as input_grid.')
    d_in = [float(d) for d in input_grid.delta]
    s_in = [int(d) for d in input_grid.dims]
    f_delta = [float(d) for d in fft_grid.delta]
    f_dims = [int(d) for d in fft_grid.dims]
    f_zero = [float(z) for z in fft_grid.zero]
    q = tuple((2 * math.pi / (d * s)) / fd for d, s, fd in zip(d_in, s_in, f_delta))
    if any(qi < 1 for qi in q):
        raise ValueError('fft_grid is not an FFT grid of input_grid: q of %s would be < 1.' % (q,))
    zp = tuple(qi * d for qi, d in zip(q, s_in))
    if any(abs(z - round(z)) > 1e-10 for z in zp):
        raise ValueError('fft_grid is not an FFT grid of input_grid: q of %s does not correspond to an integer '
                         'zeropadding.' % (q,))
    fov = tuple(fd / z for fd, z in zip(f_dims, zp))
    if any(n > int(z + 0.5) for n, z in zip(f_dims, zp)):
        raise ValueError('fft_grid is not an FFT grid of input_grid: fov of %s would be > 1 .' % (fov,))
    dummy = make_fft_grid(input_grid, q, fov)
    wrong = tuple(int(n) != m for n, m in zip(dummy.dims, f_dims))
    fov = tuple((fd + 0.5) / (d * qi) if w else f for w, f, fd, d, qi in zip(wrong, fov, f_dims, s_in, q))
    shift = tuple(z - dl * (-n / 2 + (n % 2) * 0.5) for z, dl, n in zip(f_zero, f_delta, f_dims))
    return q, fov, shift


def is_fft_grid(grid, input_grid):
    try:
        get_fft_parameters(grid, input_grid)
    except ValueError:
        return False
    return True


# ---------------------------------------------------------------------------
# Planner
# ---------------------------------------------------------------------------


def make_fourier_transform(input_grid, output_grid=None, q=1, fov=1, shift=0, planner='estimate'):
    """Choose and construct a Fourier operator (hcipy/fourier/fourier_transform.py:217-300).

    ``planner='estimate'`` (default) ranks the methods with the reference's own
    operation counts and time model, so a drop-in user gets the method the
    reference would pick (and its numerical behaviour); ``'gpu'`` ranks them with
    the GB300 cost model of this package; ``'measure'`` times each on the device.
    """
    options, expected, output_grid, (q, fov, shift) = _planned_methods(input_grid, output_grid, q, fov, shift,
                                                                        planner)
    best = min(expected, key=expected.get)
    if best == 'fft':
        return options['fft'](input_grid, q, fov, shift)
    return options[best](input_grid, output_grid)


def _planned_methods(input_grid, output_grid, q, fov, shift, planner):
    """The planner's candidates and their expected times: (classes by method, times by supported method, the
    output grid, the FFT parameters).  Without construction for the 'estimate' and 'gpu' planners."""
    options = {'mft': MatrixFourierTransform}
    try:
        from .fft import FastFourierTransform, ZoomFastFourierTransform
        options['fft'] = FastFourierTransform
        options['zft'] = ZoomFastFourierTransform
    except ImportError:
        pass
    if output_grid is not None:
        try:
            q, fov, shift = get_fft_parameters(output_grid, input_grid)
        except ValueError:
            options.pop('fft', None)
    else:
        output_grid = make_fft_grid(input_grid, q, fov, shift)

    expected = {}
    for method, ft in options.items():
        if not ft.is_supported(input_grid, output_grid):
            continue
        if planner == 'estimate':
            expected[method] = ft.compute_complexity(input_grid, output_grid).expected_execution_time
        elif planner == 'gpu':
            expected[method] = ft.gpu_execution_time(input_grid, output_grid)
        elif planner == 'measure':
            obj = ft(input_grid, q, fov, shift) if method == 'fft' else ft(input_grid, output_grid)
            a = torch.zeros(input_grid.size, dtype=torch.complex64, device='cuda')
            expected[method] = _time_device(lambda: obj.forward(a))
        else:
            raise ValueError('planner must be "estimate", "gpu" or "measure"')
    if not expected:
        raise ValueError('No Fourier transform supports these grids (unstructured grids need a naive DFT).')
    return options, expected, output_grid, (q, fov, shift)


def _time_device(fn, repeat=5):
    """Median device time of ``fn`` with CUDA events (the GPU analogue of fourier_transform.py:185-215)."""
    fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(repeat):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        times.append(s.elapsed_time(e) * 1e-3)
    return float(np.median(times))
