"""Coronagraphs: the Lyot coronagraph (hcipy/coronagraphy/lyot.py:7-122) with the Babinet chain fused into the MFT
GEMMs, and the multi-scale, vortex and vector-vortex coronagraphs (multi_scale.py, vortex.py)."""
import collections

import numpy as np
import torch

from . import _lib
from .field import Field, as_tensor
from .fourier import MatrixFourierTransform
from .optics import (AgnosticOpticalElement, OpticalElement, Apodizer, Wavefront, make_agnostic_backward,
                     make_agnostic_forward)
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
        return wavefront._carry(Field(out, e.grid))

    def _lyot_tensor(self, t, inst):
        """The fused chain on a tensor of pupil fields (..., n): one library call."""
        ft = inst.fourier_transform
        one_minus, stop = self._fused_masks(t.dtype)
        a_fwd = complex(ft._w_in_scalar) * inst.norm_factor
        a_bwd = complex(ft._w_out_scalar / (2 * np.pi)**ft.ndim) / inst.norm_factor
        out_dtype = torch.complex128 if ft.precision == 'split' else t.dtype
        return self._lyot_call(t, inst, one_minus, stop, a_fwd, a_bwd, out_dtype)

    def _lyot_call(self, t, inst, one_minus, stop, a_fwd, a_bwd, out_dtype):
        """S (E - a_bwd P^-1[a_fwd P(E) (1 - M)]) for the given masks, alphas and output dtype (hx_lyot_execute)."""
        ft = inst.fourier_transform
        t = t.detach().contiguous()
        lead = tuple(t.shape[:-1])
        batch = int(np.prod(lead)) if lead else 1
        out = torch.empty(lead + (t.shape[-1],), dtype=out_dtype, device=t.device)
        if batch == 0:
            return out
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
        wf_foc = wavefront._carry(wf_foc.electric_field - masked)
        lyot = self.prop.backward(wf_foc)
        lyot = wavefront._carry(wavefront.electric_field - lyot.electric_field)
        if self.lyot_stop is not None:
            lyot = self.lyot_stop.forward(lyot)
        return lyot

    def backward(self, wavefront):
        """lyot.py:94-122, as the reference computes it (its pupil-plane backward uses prop.forward)."""
        wf = self.lyot_stop.backward(wavefront) if self.lyot_stop is not None else wavefront
        wf_foc = self.prop.forward(wf)
        masked = self.focal_plane_mask.backward(wf_foc).electric_field
        wf_foc = wavefront._carry(wf_foc.electric_field - masked)
        pup = self.prop.backward(wf_foc)
        return wavefront._carry(wf.electric_field - pup.electric_field)


class MultiScaleCoronagraph(OpticalElement):
    """A focal-plane phase mask resolved on nested focal grids (hcipy/coronagraphy/multi_scale.py:10-161).

    Level 0 applies the mask on the q=2 FFT grid of the pupil as a Fourier filter; level i > 0 samples a window of
    ``window_size`` pixels around the centre of level i-1 ``scaling_factor`` times finer, with the part already
    applied by the coarser levels subtracted from its mask (a Tukey window tapers each level's hand-over), and
    propagates it with a forward and an inverse matrix Fourier transform at unit wavelength and focal length.
    Here each finer level is two MFT launches with the mask product fused into the first and the accumulation
    into the Lyot-plane field fused into the second (``L <- L + P^-1(M P(E))``).  The masks are built on the
    device in float64 with this package's FFT and MFT.  Lyot-plane fields follow the input bit depth.
    """

    def __init__(self, input_grid, complex_mask, lyot_stop=None, q=1024, scaling_factor=4, window_size=32):
        from scipy.signal import windows
        from .fft import FastFourierTransform, FourierFilter
        from .field import make_focal_grid
        import math
        self.input_grid = input_grid
        pupil_diameter = np.asarray(input_grid.dims, np.float64) * np.asarray(input_grid.delta, np.float64)
        if hasattr(lyot_stop, 'forward') or lyot_stop is None:
            self.lyot_stop = lyot_stop
        else:
            self.lyot_stop = Apodizer(lyot_stop)
        levels = int(math.ceil(math.log(q / 2) / math.log(scaling_factor))) + 1
        qs = [2 * scaling_factor**i for i in range(levels)]
        num_airys = [tuple(n / 2 for n in input_grid.dims)]
        for i in range(1, levels):
            num_airys.append(tuple(na * window_size / (2 * qs[i - 1] * na) for na in num_airys[i - 1]))
        self.focal_grids, self.focal_masks = [], []
        self._mfts = [None]
        dev = torch.device('cuda')
        for i in range(levels):
            focal_grid = make_focal_grid(qs[i], num_airys[i], pupil_diameter=pupil_diameter, reference_wavelength=1,
                                         focal_length=1)
            mask = np.asarray(complex_mask(focal_grid), np.complex128).ravel().copy()
            if i != levels - 1:
                w = np.outer(windows.tukey(window_size, 1, False), windows.tukey(window_size, 1, False))
                shape = (int(focal_grid.dims[1]), int(focal_grid.dims[0]))
                w = np.pad(w, tuple((n_foc - n_w) // 2 for n_foc, n_w in zip(shape, w.shape)), 'constant').ravel()
                mask *= 1 - w
            mask_t = torch.from_numpy(mask).to(dev)
            for j in range(i):
                fft = FastFourierTransform(self.focal_grids[j])
                mft = MatrixFourierTransform(focal_grid, fft.output_grid)
                mask_t = mask_t - mft.backward(fft.forward(self.focal_masks[j].data)).data
            self.focal_grids.append(focal_grid)
            self.focal_masks.append(Field(mask_t, focal_grid))
            if i == 0:
                self._filter = FourierFilter(input_grid, mask_t, qs[0])
            else:
                self._mfts.append(MatrixFourierTransform(input_grid, focal_grid.scaled(2 * np.pi)))
        self._masks = {}

    def _mask(self, i, dtype, conj):
        key = (i, dtype, conj)
        m = self._masks.get(key)
        if m is None:
            m = self.focal_masks[i].data
            m = (m.conj() if conj else m).to(dtype).contiguous().resolve_conj()
            self._masks[key] = m
        return m

    def _propagate(self, e, conj):
        """L = F(E) + sum_i P_i^-1(M_i P_i(E)) (conj: the conjugate masks and the backward filter)."""
        lyot = (self._filter.backward(e) if conj else self._filter.forward(e)).data
        # Fraunhofer at unit wavelength and focal length: norm 1/(i f lambda) = -i (fraunhofer.py:32-38)
        norm = -1j
        for i in range(1, len(self.focal_masks)):
            ft = self._mfts[i]
            a_fwd = complex(ft._w_in_scalar) * norm
            a_bwd = complex(ft._w_out_scalar / (2 * np.pi)**2) / norm
            focal = ft._run(e, ft.input_grid, ft.output_grid, _lib.HX_FORWARD, a_fwd, epilogue=_lib.HX_EPI_MUL,
                            mask=self._mask(i, e.dtype, conj)).data
            # lyot <- lyot - (-a_bwd) M1b focal M2b: the Babinet epilogue without a stop accumulates in place
            ft._run(focal, ft.output_grid, ft.input_grid, _lib.HX_BACKWARD, -a_bwd, epilogue=_lib.HX_EPI_BABINET,
                    src=lyot, out=lyot)
        return lyot

    def forward(self, wavefront):
        """multi_scale.py:95-128."""
        e = as_tensor(wavefront.electric_field).contiguous()
        lyot = wavefront._carry(Field(self._propagate(e, False), self.input_grid))
        if self.lyot_stop is not None:
            lyot = self.lyot_stop.forward(lyot)
        return lyot

    def backward(self, wavefront):
        """multi_scale.py:130-161: the same chain with the conjugate masks."""
        if self.lyot_stop is not None:
            wavefront = self.lyot_stop.backward(wavefront)
        e = as_tensor(wavefront.electric_field).contiguous()
        return wavefront._carry(Field(self._propagate(e, True), self.input_grid))


class VortexCoronagraph(MultiScaleCoronagraph):
    """A scalar vortex of ``charge`` (hcipy/coronagraphy/vortex.py:12-15): the mask exp(i charge theta), zero at
    the singularity, on the multi-scale focal grids."""

    def __init__(self, input_grid, charge, lyot_stop=None, q=1024, scaling_factor=4, window_size=32):
        self.charge = charge

        def complex_mask(grid):
            x, y = grid.points_list()
            centre = np.hypot(x, y) <= 0.5e-9  # make_circular_aperture(1e-9), boundary inclusive
            return np.exp(1j * charge * np.arctan2(y, x)) * (1 - centre)

        MultiScaleCoronagraph.__init__(self, input_grid, complex_mask, lyot_stop, q, scaling_factor, window_size)


class VectorVortexCoronagraph(AgnosticOpticalElement):
    """A vector vortex of ``charge`` (hcipy/coronagraphy/vortex.py:17-246): a linear retarder in the focal plane whose
    fast axis turns as charge / 2 times the azimuth, resolved on the multi-scale focal grids; same arguments.

    The retarder's Jones matrix (polarization.py:141-160, retardance G, fast-axis angle a)
    j11 = e^{iG/2} cos^2 a + e^{-iG/2} sin^2 a,  j12 = j21 = (e^{iG/2} - e^{-iG/2}) cos a sin a,
    j22 = e^{iG/2} sin^2 a + e^{-iG/2} cos^2 a
    is symmetric, and each step of the multi-scale construction (the central pinhole, the Tukey windows, the
    subtraction of the coarser levels) and of the propagation acts on every entry alone.  The coronagraph is
    therefore three scalar multi-scale coronagraphs C11, C12, C22, one per distinct entry: an unpolarised field E
    gives the Lyot-plane Jones matrix [[C11 E, C12 E], [C12 E, C22 E]] (the reference's E times the identity,
    Stokes vector (1, 0, 0, 0)); a polarised wavefront's (2, 2, n) Jones matrix gives L_ik = sum_j C_ij(E_jk), each
    C applied to a batch of two fields.  ``backward`` applies the conjugate masks, which for a symmetric J is the
    conjugate transpose the reference applies.  The propagation is at unit wavelength (the masks are in lambda/D);
    the retardance may depend on the wavelength.
    """

    def __init__(self, charge, lyot_stop=None, phase_retardation=np.pi, q=1024, scaling_factor=4, window_size=32):
        self.charge = charge
        if hasattr(lyot_stop, 'forward') or lyot_stop is None:
            self.lyot_stop = lyot_stop
        else:
            self.lyot_stop = Apodizer(lyot_stop)
        self.phase_retardation = phase_retardation
        self.q = q
        self.scaling_factor = scaling_factor
        self.window_size = window_size
        self._entries = collections.OrderedDict()
        AgnosticOpticalElement.__init__(self)

    def _jones_entry(self, retardance, which):
        charge = self.charge

        def mask(grid):
            x, y = grid.points_list()
            a = charge / 2 * np.arctan2(y, x)
            plus, minus = np.exp(1j * retardance / 2), np.exp(-1j * retardance / 2)
            if which == 'j11':
                j = plus * np.cos(a)**2 + minus * np.sin(a)**2
            elif which == 'j22':
                j = plus * np.sin(a)**2 + minus * np.cos(a)**2
            else:
                j = (plus - minus) * np.cos(a) * np.sin(a)
            centre = np.hypot(x, y) <= 0.5e-9  # make_circular_aperture(1e-9), boundary inclusive
            return j * (1 - centre)
        return mask

    def make_instance(self, instance_data, input_grid, output_grid, wavelength):
        from .field import grid_key
        retardance = float(self.evaluate_parameter(self.phase_retardation, input_grid, output_grid, wavelength))
        key = (grid_key(input_grid), retardance)
        entries = self._entries.get(key)
        if entries is None:
            # the same retardance at another wavelength reuses the three coronagraphs; at most as many sets as
            # the instance cache holds, first in first out
            entries = tuple(MultiScaleCoronagraph(input_grid, self._jones_entry(retardance, w), None, self.q,
                                                  self.scaling_factor, self.window_size)
                            for w in ('j11', 'j12', 'j22'))
            if len(self._entries) >= self._max_in_cache:
                self._entries.popitem(last=False)
            self._entries[key] = entries
        instance_data.entries = entries

    def get_input_grid(self, output_grid, wavelength):
        return output_grid

    def get_output_grid(self, input_grid, wavelength):
        return input_grid

    def _propagate(self, entries, wavefront, conj):
        c11, c12, c22 = entries
        e = as_tensor(wavefront.electric_field).contiguous()
        if wavefront.is_polarized:
            stokes = wavefront.input_stokes_vector
            row0 = c11._propagate(e[0], conj) + c12._propagate(e[1], conj)
            row1 = c12._propagate(e[0], conj) + c22._propagate(e[1], conj)
            out = torch.stack((row0, row1))
        else:
            if e.dim() != 1:
                raise ValueError('The vector vortex takes one scalar field or a polarised wavefront.')
            stokes = (1, 0, 0, 0)
            j11, j12, j22 = (c._propagate(e, conj) for c in entries)
            out = torch.stack((torch.stack((j11, j12)), torch.stack((j12, j22))))
        return Wavefront(Field(out, wavefront.electric_field.grid), wavefront.wavelength, stokes)

    @make_agnostic_forward
    def forward(self, instance_data, wavefront):
        """vortex.py:160-202."""
        lyot = self._propagate(instance_data.entries, wavefront, False)
        if self.lyot_stop is not None:
            lyot = self.lyot_stop.forward(lyot)
        return lyot

    @make_agnostic_backward
    def backward(self, instance_data, wavefront):
        """vortex.py:204-246."""
        if self.lyot_stop is not None:
            wavefront = self.lyot_stop.backward(wavefront)
        return self._propagate(instance_data.entries, wavefront, True)
