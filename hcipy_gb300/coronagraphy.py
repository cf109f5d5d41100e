"""Lyot coronagraph (hcipy/coronagraphy/lyot.py:7-122) with the Babinet chain fused into the MFT GEMMs."""
import numpy as np
import torch

from . import _lib
from .field import Field, as_tensor
from .fourier import MatrixFourierTransform
from .optics import OpticalElement, Apodizer, Wavefront
from .propagation import FraunhoferPropagator


class LyotCoronagraph(OpticalElement):
    """A Lyot coronagraph with a small focal-plane mask, propagated with Babinet's principle.

    forward (lyot.py:66-92):  E_f = P(E);  E_f <- E_f - M E_f;  L = P^-1(E_f);  L <- E - L;  L <- S L.

    When the focal-plane mask and the Lyot stop are fields and the propagator
    uses a matrix Fourier transform, the chain is one library call
    (``hx_lyot_execute``): the mask product ``E_f (1 - M)`` is the epilogue of
    the forward MFT's last GEMM, and ``S (E - L)`` the epilogue of the inverse
    MFT's last GEMM.  With ``precision='split'`` the focal-plane field stays in
    float-float between the transforms and the Lyot plane is returned as
    complex128.  Other masks (optical elements) run the same steps one
    operator at a time.
    """

    def __init__(self, input_grid, focal_plane_mask, lyot_stop=None, focal_length=1, focal_plane_mask_grid=None,
                 precision='fp32'):
        if isinstance(focal_plane_mask, OpticalElement):
            if focal_plane_mask_grid is None:
                raise ValueError('Could not determine the input grid of the focal plane mask. Please pass '
                                 'focal_plane_mask_grid explicitly.')
            grid = focal_plane_mask_grid
            self.focal_plane_mask = focal_plane_mask
            self._fpm_field = None
        else:
            grid = focal_plane_mask.grid if focal_plane_mask_grid is None else focal_plane_mask_grid
            self.focal_plane_mask = Apodizer(focal_plane_mask)
            self._fpm_field = focal_plane_mask
        self._stop_field = None
        if lyot_stop is not None and not isinstance(lyot_stop, OpticalElement):
            self._stop_field = lyot_stop
            lyot_stop = Apodizer(lyot_stop)
        self.lyot_stop = lyot_stop
        self.prop = FraunhoferPropagator(input_grid, grid, focal_length=focal_length, precision=precision)
        self._masks = {}

    def _fused_masks(self, dtype):
        if self.prop.precision == 'split':
            dtype = torch.complex64
        m = self._masks.get(dtype)
        if m is None:
            fpm = as_tensor(self._fpm_field).to(dtype).reshape(-1)
            one_minus = (1 - fpm).contiguous()
            stop = None
            if self._stop_field is not None:
                stop = as_tensor(self._stop_field).to(dtype).reshape(-1).contiguous()
            m = (one_minus, stop)
            self._masks[dtype] = m
        return m

    def _can_fuse(self, inst):
        return (self._fpm_field is not None and (self.lyot_stop is None or self._stop_field is not None)
                and isinstance(inst.fourier_transform, MatrixFourierTransform) and not callable(self._fpm_field))

    def forward(self, wavefront):
        inst = self.prop.get_instance_data(wavefront.grid, None, wavefront.wavelength)
        if not self._can_fuse(inst):
            return self._forward_unfused(wavefront)
        e = wavefront.electric_field
        t = as_tensor(e)
        if torch.is_grad_enabled() and t.requires_grad:
            from .autograd import LyotFunction
            out = LyotFunction.apply(t, self, inst)
        else:
            out = self._lyot_tensor(t, inst)
        return Wavefront(Field(out, e.grid), wavefront.wavelength)

    def _lyot_tensor(self, t, inst):
        """The fused chain on a tensor of pupil fields (..., n): one library call."""
        ft = inst.fourier_transform
        t = t.detach().contiguous()
        split = ft.precision == 'split'
        one_minus, stop = self._fused_masks(t.dtype)
        a_fwd = complex(ft._w_in_scalar) * inst.norm_factor
        a_bwd = complex(ft._w_out_scalar / (2 * np.pi)**ft.ndim) / inst.norm_factor
        lead = tuple(t.shape[:-1])
        batch = int(np.prod(lead)) if lead else 1
        out = torch.empty(lead + (t.shape[-1],), dtype=torch.complex128 if split else t.dtype, device=t.device)
        plan = ft._plan(t.dtype)
        lib = _lib.lib()
        nbytes = int(lib.hx_lyot_workspace_bytes(plan.handle, None, batch))
        ws = _lib.workspace(nbytes, t.device)
        rc = lib.hx_lyot_execute(plan.handle, None, batch, _lib.dptr(t), _lib.dtype_code(t.dtype),
                                 _lib.dptr(one_minus), None if stop is None else _lib.dptr(stop),
                                 a_fwd.real, a_fwd.imag, a_bwd.real, a_bwd.imag, 0.0, 0.0,
                                 _lib.dptr(out), _lib.dtype_code(out.dtype), None, _lib.HX_C64,
                                 _lib.dptr(ws), nbytes, _lib.stream_handle())
        _lib.check(rc, 'hx_lyot_execute')
        return out

    def _forward_unfused(self, wavefront):
        wf_foc = self.prop.forward(wavefront)
        masked = self.focal_plane_mask.forward(wf_foc).electric_field
        wf_foc = Wavefront(wf_foc.electric_field - masked, wavefront.wavelength)
        lyot = self.prop.backward(wf_foc)
        lyot = Wavefront(wavefront.electric_field - lyot.electric_field, wavefront.wavelength)
        if self.lyot_stop is not None:
            lyot = self.lyot_stop.forward(lyot)
        return lyot

    def backward(self, wavefront):
        """lyot.py:94-122, as the reference computes it (its pupil-plane backward uses prop.forward)."""
        wf = self.lyot_stop.backward(wavefront) if self.lyot_stop is not None else wavefront
        wf_foc = self.prop.forward(wf)
        masked = self.focal_plane_mask.backward(wf_foc).electric_field
        wf_foc = Wavefront(wf_foc.electric_field - masked, wavefront.wavelength)
        pup = self.prop.backward(wf_foc)
        return Wavefront(wf.electric_field - pup.electric_field, wavefront.wavelength)
