"""FFT-family operators on the device: FastFourierTransform, ChirpZTransform,
ZoomFastFourierTransform and FourierFilter (hcipy/fourier/*).

Plans hold float64-derived constant tables (twiddles, chirps, phase factors,
transfer functions) in the field's element type; every execute is one to three
launches of the shared-memory line-FFT kernel.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .field import Field, as_tensor, complex_dtype_for
from .fourier import (FourierTransform, ComputationalComplexity, make_fft_grid, get_fft_parameters, _is_cartesian,
                      _prepare_input, cost_model, reference_seconds)


def _grid_axes(grid):
    return [np.asarray(c, np.float64) for c in grid.separated_coords]


class _Plan(object):
    """Owner of one C plan handle."""

    def __init__(self, handle, destroy):
        self.handle = handle
        self._destroy = destroy

    def __del__(self):
        try:
            if self.handle:
                self._destroy(self.handle)
        except Exception:
            pass


# ---------------------------------------------------------------------------
# FastFourierTransform (hcipy/fourier/fast_fourier_transform.py:188-482)
# ---------------------------------------------------------------------------


class FastFourierTransform(FourierTransform):
    """Zero-padded FFT with cropping and output shift, on the device.

    The reference's ``emulate_fftshifts`` option trades accuracy for speed on the
    CPU; here the fftshifts are exact index shifts inside the kernel, so the flag
    is accepted and has no effect.
    """

    def __init__(self, input_grid, q=1, fov=1, shift=0, emulate_fftshifts=None):
        if not input_grid.is_regular:
            raise ValueError('The input_grid must be regular.')
        if not _is_cartesian(input_grid):
            raise ValueError('The input_grid must be Cartesian.')
        q_check = (q,) if np.isscalar(q) else q
        fov_check = (fov,) if np.isscalar(fov) else fov
        if any(qi < 1 for qi in q_check):
            raise ValueError('The amount of zeropadding (q) must be larger than 1.')
        if any(fi < 0 for fi in fov_check):
            raise ValueError('The amount of cropping (fov) must be positive.')
        if input_grid.ndim not in (1, 2):
            raise ValueError('hcipy_gb300 computes one- and two-dimensional FFTs.')
        self.input_grid = input_grid
        self.emulate_fftshifts = emulate_fftshifts
        self.ndim = input_grid.ndim
        self.output_grid = make_fft_grid(input_grid, q, fov, shift)
        self.internal_grid = make_fft_grid(input_grid, q, 1)
        n_in = [int(d) for d in input_grid.dims]
        n_int = [int(d) for d in self.internal_grid.dims]
        n_out = [int(d) for d in self.output_grid.dims]
        if any(o > i for o, i in zip(n_out, n_int)):
            raise ValueError('The amount of cropping (fov) must be smaller than 1.')
        self.shape_in = tuple(n_in[::-1])
        self.shape_out = tuple(n_out[::-1])
        self.internal_shape = tuple(n_int[::-1])
        # Cutouts (fast_fourier_transform.py:261-275), per axis, x first.
        self._n_in, self._n_int, self._n_out = n_in, n_int, n_out
        self._c_in = [int(N / 2) - int(n / 2) for N, n in zip(n_int, n_in)]
        self._c_out = [int(N / 2) - int(n / 2) for N, n in zip(n_int, n_out)]
        # shift_input (:279-297), separable: exp(-i c_d (k_d - k_d[n/2])) per axis, times the weight.
        delta = np.asarray(input_grid.delta, np.float64)
        zero = np.asarray(input_grid.zero, np.float64)
        center = zero + delta * (np.asarray(n_in) // 2)
        ks = _grid_axes(self.output_grid)
        self._post = [np.exp(-1j * c * (k - k[len(k) // 2])) for c, k in zip(center, ks)]
        self._scale = float(np.prod(delta))
        # shift_output (:301-305).
        shift_v = np.ones(self.ndim) * shift
        if np.allclose(shift_v, 0):
            self._pre = [None] * self.ndim
        else:
            xs = _grid_axes(input_grid)
            self._pre = [np.exp(-1j * s * x) for s, x in zip(shift_v, xs)]
        self._plans = {}

    def _plan(self, cdt):
        plan = self._plans.get(cdt)
        if plan is not None:
            return plan
        lib = _lib.lib()
        keep = []
        dims = []
        for v in (self._n_in, self._n_int, self._n_out, self._c_in, self._c_out):
            buf, p = _lib.iarr(v)
            keep.append(buf)
            dims.append(p)
        pre_ptrs, post_ptrs = [], []
        for arr in self._pre:
            buf, p = _lib.carr(arr)
            keep.append(buf)
            pre_ptrs.append(p)
        for arr in self._post:
            buf, p = _lib.carr(arr)
            keep.append(buf)
            post_ptrs.append(p)
        pre_arr, pre_pp = _lib.ptr_array(pre_ptrs)
        post_arr, post_pp = _lib.ptr_array(post_ptrs)
        handle = ctypes.c_void_p()
        rc = lib.hx_fft_plan_create(self.ndim, *dims, pre_pp, post_pp, self._scale, 0.0, _lib.dtype_code(cdt),
                                    _lib.stream_handle(), ctypes.byref(handle))
        _lib.check(rc, 'hx_fft_plan_create')
        plan = _Plan(handle, lib.hx_fft_plan_destroy)
        self._plans[cdt] = plan
        return plan

    def _run(self, field, src_grid, dst_grid, direction):
        t = _prepare_input(field, src_grid)
        batch_shape = tuple(t.shape[:-1])
        batch = int(np.prod(batch_shape)) if batch_shape else 1
        out = torch.empty(batch_shape + (dst_grid.size,), dtype=t.dtype, device=t.device)
        if batch > 0:
            lib = _lib.lib()
            plan = self._plan(t.dtype)
            nbytes = lib.hx_fft_workspace_bytes(plan.handle, direction, batch)
            ws = _lib.workspace(nbytes, t.device)
            rc = lib.hx_fft_execute(plan.handle, direction, batch, _lib.dptr(t), _lib.dptr(out), _lib.dptr(ws),
                                    nbytes, _lib.stream_handle())
            _lib.check(rc, 'hx_fft_execute')
        return Field(out, dst_grid)

    def forward(self, field):
        """fast_fourier_transform.py:324-365."""
        return self._run(field, self.input_grid, self.output_grid, _lib.HX_FORWARD)

    def backward(self, field):
        """fast_fourier_transform.py:367-406."""
        return self._run(field, self.output_grid, self.input_grid, _lib.HX_BACKWARD)

    @property
    def adjoint_scale(self):
        """forward = scale Post Crop F Pad Pre with unit-modulus phase factors and the unnormalised DFT F, whose
        adjoint F^H is N times the normalised inverse; ``backward`` divides by scale and N, so the adjoint of
        ``forward`` is scale^2 N ``backward``.  Not part of the reference API."""
        return self._scale**2 * float(np.prod(self._n_int))

    def adjoint(self, field):
        """The conjugate transpose of ``forward``; not part of the reference API."""
        out = self.backward(field)
        return Field(out.data * self.adjoint_scale, self.input_grid)

    @classmethod
    def check_if_supported(cls, input_grid, output_grid):
        get_fft_parameters(output_grid, input_grid)
        if input_grid.ndim not in (1, 2):
            raise ValueError('hcipy_gb300 computes one- and two-dimensional FFTs.')

    @classmethod
    def compute_complexity(cls, input_grid, output_grid):
        """Operation count of fast_fourier_transform.py:427-482 and a GB300 time estimate."""
        q, _, shift = get_fft_parameters(output_grid, input_grid)
        shape = tuple(n * qq for n, qq in zip(input_grid.dims, q))
        n_int = math.prod(shape)
        n_in = input_grid.size
        n_out = output_grid.size
        cmul = 0.5 * n_int * math.log2(n_int) + n_out + (0 if np.allclose(shift, 0) else n_in)
        cadd = n_int * math.log2(n_int)
        mults = 4 * cmul
        adds = 2 * cmul + 2 * cadd
        return ComputationalComplexity(mults, adds, reference_seconds('fft', mults + adds))

    @classmethod
    def gpu_execution_time(cls, input_grid, output_grid):
        """GB300 estimate: one line-FFT launch per axis, bound by HBM traffic or butterflies."""
        q, _, _ = get_fft_parameters(output_grid, input_grid)
        n_int = math.prod(n * qq for n, qq in zip(input_grid.dims, q))
        ndim = input_grid.ndim
        n_mid = int(np.asarray(input_grid.dims)[1]) * int(output_grid.dims[0]) if ndim == 2 else 0
        return cost_model.fft_seconds(n_int, input_grid.size, output_grid.size, passes=ndim, n_mid=n_mid)


# ---------------------------------------------------------------------------
# Chirp-Z transform (hcipy/fourier/chirp_z_transform.py:7-105)
# ---------------------------------------------------------------------------


class ChirpZTransform(object):
    """X_k = sum_n x(n) z_k^-n, z_k = a w^-k, along the last axis, by Bluestein's algorithm in one launch."""

    def __init__(self, n, m, w, a):
        self.n = int(n)
        self.m = int(m)
        self.w = complex(w)
        self.a = complex(a)
        self._plans = {}

    def _plan(self, cdt, pre=None, post=None):
        key = (cdt, id(pre), id(post))
        plan = self._plans.get(key)
        if plan is None:
            lib = _lib.lib()
            bpre, ppre = _lib.carr(pre)
            bpost, ppost = _lib.carr(post)
            handle = ctypes.c_void_p()
            rc = lib.hx_czt_plan_create(self.n, self.m, self.w.real, self.w.imag, self.a.real, self.a.imag, ppre,
                                        ppost, _lib.dtype_code(cdt), _lib.stream_handle(), ctypes.byref(handle))
            _lib.check(rc, 'hx_czt_plan_create')
            plan = _Plan(handle, lib.hx_czt_plan_destroy)
            self._plans[key] = plan
        return plan

    def __call__(self, x):
        t = as_tensor(x)
        cdt = complex_dtype_for(t.dtype)
        t = t.to(cdt).contiguous()
        if t.shape[-1] != self.n:
            raise ValueError('The last axis must have %d points.' % self.n)
        lead = tuple(t.shape[:-1])
        lines = int(np.prod(lead)) if lead else 1
        out = torch.empty(lead + (self.m,), dtype=cdt, device=t.device)
        if lines:
            plan = self._plan(cdt)
            rc = _lib.lib().hx_czt_execute(plan.handle, lines, 1, _lib.dptr(t), self.n, 1, 0, _lib.dptr(out), self.m,
                                           1, 0, _lib.stream_handle())
            _lib.check(rc, 'hx_czt_execute')
        return out


# ---------------------------------------------------------------------------
# Zoom FFT (hcipy/fourier/zoom_fast_fourier_transform.py:10-219)
# ---------------------------------------------------------------------------


class ZoomFastFourierTransform(FourierTransform):
    """Per-axis chirp-Z transforms between regular grids; weights and shifts are folded into the chirps."""

    def __init__(self, input_grid, output_grid):
        self.check_if_supported(input_grid, output_grid)
        self.input_grid = input_grid
        self.output_grid = output_grid
        self.ndim = input_grid.ndim
        self._plans = {}

    def _axis_plans(self, cdt, inverse):
        key = (cdt, inverse)
        if key in self._plans:
            return self._plans[key]
        gi, go = (self.output_grid, self.input_grid) if inverse else (self.input_grid, self.output_grid)
        d_in = np.asarray(gi.delta, np.float64)
        z_in = np.asarray(gi.zero, np.float64)
        d_out = np.asarray(go.delta, np.float64)
        z_out = np.asarray(go.zero, np.float64)
        n_in = [int(d) for d in gi.dims]
        n_out = [int(d) for d in go.dims]
        sign = 1 if inverse else -1
        weight = (float(np.prod(d_in)) / (2 * math.pi)**self.ndim) if inverse else float(np.prod(d_in))
        plans = []
        lib = _lib.lib()
        for ax in range(self.ndim):
            w = np.exp(sign * 1j * d_out[ax] * d_in[ax])
            a = np.exp(-sign * 1j * z_out[ax] * d_in[ax])
            coords_out = z_out[ax] + d_out[ax] * np.arange(n_out[ax])
            post = np.exp(sign * 1j * coords_out * z_in[ax])
            pre = np.full(n_in[ax], weight if ax == 0 else 1.0, dtype=np.complex128)
            bpre, ppre = _lib.carr(pre)
            bpost, ppost = _lib.carr(post)
            handle = ctypes.c_void_p()
            rc = lib.hx_czt_plan_create(n_in[ax], n_out[ax], w.real, w.imag, a.real, a.imag, ppre, ppost,
                                        _lib.dtype_code(cdt), _lib.stream_handle(), ctypes.byref(handle))
            _lib.check(rc, 'hx_czt_plan_create')
            plans.append(_Plan(handle, lib.hx_czt_plan_destroy))
        self._plans[key] = (plans, n_in, n_out)
        return self._plans[key]

    def _run(self, field, src, dst, inverse):
        t = _prepare_input(field, src)
        lead = tuple(t.shape[:-1])
        batch = int(np.prod(lead)) if lead else 1
        out = torch.empty(lead + (dst.size,), dtype=t.dtype, device=t.device)
        if batch == 0:
            return Field(out, dst)
        plans, n_in, n_out = self._axis_plans(t.dtype, inverse)
        lib = _lib.lib()
        s = _lib.stream_handle()
        if self.ndim == 1:
            rc = lib.hx_czt_execute(plans[0].handle, batch, 1, _lib.dptr(t), n_in[0], 1, 0, _lib.dptr(out), n_out[0],
                                    1, 0, s)
            _lib.check(rc, 'hx_czt_execute')
            return Field(out, dst)
        nx, ny = n_in
        mx, my = n_out
        mid = torch.empty(lead + (ny * mx,), dtype=t.dtype, device=t.device)
        # along x: ny rows per field
        rc = lib.hx_czt_execute(plans[0].handle, ny, batch, _lib.dptr(t), nx, 1, nx * ny, _lib.dptr(mid), mx, 1,
                                ny * mx, s)
        _lib.check(rc, 'hx_czt_execute')
        # along y: mx columns per field
        rc = lib.hx_czt_execute(plans[1].handle, mx, batch, _lib.dptr(mid), 1, mx, ny * mx, _lib.dptr(out), 1, mx,
                                my * mx, s)
        _lib.check(rc, 'hx_czt_execute')
        return Field(out, dst)

    def forward(self, field):
        """zoom_fast_fourier_transform.py:69-93."""
        return self._run(field, self.input_grid, self.output_grid, False)

    def backward(self, field):
        """zoom_fast_fourier_transform.py:95-119."""
        return self._run(field, self.output_grid, self.input_grid, True)

    @property
    def adjoint_scale(self):
        """Both directions are exact DFTs on the grids: forward = w_in sum E exp(-i u x), backward = w_out/(2 pi)^d
        sum F exp(+i u x), so the adjoint of ``forward`` is w_in (2 pi)^d / w_out ``backward``.  Not part of the
        reference API."""
        w_in = float(np.prod(np.asarray(self.input_grid.delta, np.float64)))
        w_out = float(np.prod(np.asarray(self.output_grid.delta, np.float64)))
        return w_in * (2 * math.pi)**self.ndim / w_out

    def adjoint(self, field):
        """The conjugate transpose of ``forward``; not part of the reference API."""
        return Field(self.backward(field).data * self.adjoint_scale, self.input_grid)

    @classmethod
    def check_if_supported(cls, input_grid, output_grid):
        if not input_grid.is_regular or not _is_cartesian(input_grid):
            raise ValueError('The input grid should be regularly spaced in Cartesian coordinates.')
        if not output_grid.is_regular or not _is_cartesian(output_grid):
            raise ValueError('The output grid should be regularly spaced in Cartesian coordinates.')
        if input_grid.ndim != output_grid.ndim:
            raise ValueError('The input_grid must have the same dimensions as the output_grid.')
        if input_grid.ndim not in (1, 2):
            raise ValueError('hcipy_gb300 computes one- and two-dimensional zoom FFTs.')

    @classmethod
    def compute_complexity(cls, input_grid, output_grid):
        """Operation count and predicted time as the reference planner computes them
        (zoom_fast_fourier_transform.py:147-219; its CZT length is scipy's next_fast_len)."""
        import scipy.fft
        cls.check_if_supported(input_grid, output_grid)
        cmul = input_grid.size
        cadd = 0
        ins = [int(d) for d in np.asarray(input_grid.shape)]
        outs = [int(d) for d in np.asarray(output_grid.shape)]
        for i in range(len(ins)):
            L = scipy.fft.next_fast_len(ins[i] + outs[i] - 1)
            per = math.prod(outs[:i]) * math.prod(ins[i + 1:])
            before = math.prod(outs[:i]) * math.prod(ins[i:])
            after = math.prod(outs[:i + 1]) * math.prod(ins[i + 1:])
            cmul += before + 0.5 * L * per * math.log2(L) + L * per + 0.5 * L * per * math.log2(L) + 2 * after
            cadd += 2 * L * per * math.log2(L)
        mults = 4 * cmul
        adds = 2 * cmul + 2 * cadd
        return ComputationalComplexity(mults, adds, reference_seconds('zfft', mults + adds))

    @classmethod
    def gpu_execution_time(cls, input_grid, output_grid):
        """GB300 estimate: one chirp-Z launch per axis (power-of-two Bluestein length)."""
        cls.check_if_supported(input_grid, output_grid)
        secs = 0
        ins = [int(d) for d in input_grid.dims]
        outs = [int(d) for d in output_grid.dims]
        for i in range(input_grid.ndim):
            L = 1 << int(math.ceil(math.log2(ins[i] + outs[i] - 1)))
            per = math.prod(outs[:i]) * math.prod(ins[i + 1:])
            before = math.prod(outs[:i]) * math.prod(ins[i:])
            after = math.prod(outs[:i + 1]) * math.prod(ins[i + 1:])
            secs += cost_model.fft_seconds(2 * L * per, before, after, passes=1)
        return secs


# ---------------------------------------------------------------------------
# Fourier filter (hcipy/fourier/fourier_operations.py:8-151)
# ---------------------------------------------------------------------------


class FourierFilter(object):
    """pad -> FFT -> x transfer function -> IFFT -> crop, with the multiply fused into the column pass.

    ``transfer_function`` is a Field generator or a Field on the internal grid
    (centred order, as in the reference), or, with ``fft_order=True``, a device
    tensor already in FFT order.
    """

    def __init__(self, input_grid, transfer_function, q=1, fft_order=False):
        fft = FastFourierTransform(input_grid, q)
        self.input_grid = input_grid
        self.internal_grid = fft.output_grid
        self.shape_in = input_grid.shape
        self.transfer_function = transfer_function
        self._fft_order = fft_order
        self._n = [int(d) for d in input_grid.dims]
        self._N = [int(d) for d in self.internal_grid.dims]
        self._c = [int(N / 2) - int(n / 2) for N, n in zip(self._N, self._n)]
        self._plans = {}

    def _tf_tensor(self, cdt):
        tf = self.transfer_function
        if callable(tf) and not isinstance(tf, (Field, torch.Tensor, np.ndarray)):
            tf = tf(self.internal_grid)
        t = as_tensor(tf).to(cdt)
        if not self._fft_order:
            shape = tuple(self._N[::-1])
            t = torch.fft.ifftshift(t.reshape(shape), dim=tuple(range(-len(shape), 0)))
        return t.contiguous().reshape(-1)

    def _plan(self, cdt):
        plan = self._plans.get(cdt)
        if plan is None:
            lib = _lib.lib()
            tf = self._tf_tensor(cdt)
            keep = []
            ptrs = []
            for v in (self._n, self._N, self._c):
                buf, p = _lib.iarr(v)
                keep.append(buf)
                ptrs.append(p)
            handle = ctypes.c_void_p()
            rc = lib.hx_filter_plan_create(len(self._n), *ptrs, _lib.dptr(tf), _lib.dtype_code(cdt),
                                           _lib.stream_handle(), ctypes.byref(handle))
            _lib.check(rc, 'hx_filter_plan_create')
            plan = _Plan(handle, lib.hx_filter_plan_destroy)
            self._plans[cdt] = plan
        return plan

    def _operation(self, field, adjoint):
        t = _prepare_input(field, self.input_grid)
        lead = tuple(t.shape[:-1])
        batch = int(np.prod(lead)) if lead else 1
        out = torch.empty_like(t)
        if batch:
            lib = _lib.lib()
            plan = self._plan(t.dtype)
            nbytes = lib.hx_filter_workspace_bytes(plan.handle, batch)
            ws = _lib.workspace(nbytes, t.device)
            rc = lib.hx_filter_execute(plan.handle, 1 if adjoint else 0, batch, _lib.dptr(t), _lib.dptr(out),
                                       _lib.dptr(ws), nbytes, _lib.stream_handle())
            _lib.check(rc, 'hx_filter_execute')
        return Field(out, self.input_grid)

    def forward(self, field):
        """fourier_operations.py:59-72."""
        return self._operation(field, False)

    def backward(self, field):
        """fourier_operations.py:74-87 (adjoint filter)."""
        return self._operation(field, True)
