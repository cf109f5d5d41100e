"""Propagators (hcipy/propagation) on the device."""
import numpy as np
import torch

from . import _lib
from .field import Field, as_tensor
from .fourier import make_fourier_transform, MatrixFourierTransform
from .optics import AgnosticOpticalElement, make_agnostic_forward, make_agnostic_backward


def _adjoint_scale(ft):
    """c with forward^H = c backward for the FFT-family transforms the planner may pick."""
    scale = getattr(ft, 'adjoint_scale', None)
    if scale is None:
        raise NotImplementedError('gradients through a %s are not implemented' % type(ft).__name__)
    return scale


def _adjoint_of_forward(ft):
    c = _adjoint_scale(ft)
    return lambda g: ft.backward(g).data * c


def _filter_apply(ff, wavefront, adjoint):
    """The Fourier filter (or, with adjoint, its backward: the conjugate transfer function, which is the exact
    adjoint of the filter) on the wavefront's field, differentiable when the field requires grad."""
    e = wavefront.electric_field
    fwd, adj = (ff.backward, ff.forward) if adjoint else (ff.forward, ff.backward)
    if _differentiable(e):
        from .autograd import linear_apply
        res = linear_apply(e.data, lambda t: fwd(t).data, lambda g: adj(g).data)
        return wavefront._carry(Field(res, e.grid))
    return wavefront._carry(fwd(e))


def _differentiable(field):
    """True when autograd records operations on this field's tensor."""
    t = field.data if isinstance(field, Field) else field
    return torch.is_grad_enabled() and isinstance(t, torch.Tensor) and t.requires_grad


class FraunhoferPropagator(AgnosticOpticalElement):
    """A perfect lens from its front to its back focal plane (hcipy/propagation/fraunhofer.py:7-88).

    ``precision`` ('fp32' or 'split') and ``schedule`` ('latency' or 'throughput')
    are forwarded to the matrix Fourier transform when the planner picks one.
    """

    def __init__(self, input_grid, output_grid, focal_length=1, precision='fp32', schedule='latency'):
        self._input_grid = input_grid
        self._output_grid = output_grid
        self._focal_length = focal_length
        self.precision = precision
        self.schedule = schedule
        AgnosticOpticalElement.__init__(self, grid_dependent=True, wavelength_dependent=True)

    def make_instance(self, instance_data, input_grid, output_grid, wavelength):
        # fraunhofer.py:32-38.
        focal_length = self.evaluate_parameter(self.focal_length, input_grid, output_grid, wavelength)
        instance_data.uv_grid = output_grid.scaled(2 * np.pi / (focal_length * wavelength))
        ft = make_fourier_transform(input_grid, instance_data.uv_grid)
        if isinstance(ft, MatrixFourierTransform) and (self.precision != 'fp32' or self.schedule != 'latency'):
            ft = MatrixFourierTransform(input_grid, instance_data.uv_grid, precision=self.precision,
                                        schedule=self.schedule)
        instance_data.fourier_transform = ft
        instance_data.norm_factor = 1 / (1j * focal_length * wavelength)

    @property
    def focal_length(self):
        return self._focal_length

    @focal_length.setter
    def focal_length(self, focal_length):
        self._focal_length = focal_length
        self.clear_cache()

    def get_input_grid(self, output_grid, wavelength):
        return self._input_grid

    def get_output_grid(self, input_grid, wavelength):
        return self._output_grid

    def phase_screen_fusable(self, t, screen, wavelength=1):
        """Whether ``forward_phase_screen`` applies to these device tensors (checks only, no launch)."""
        inst = self.get_instance_data(self._input_grid, None, wavelength)
        ft = inst.fourier_transform
        if not isinstance(ft, MatrixFourierTransform) or ft.precision != 'split':
            return False
        if t.dtype != torch.complex64 or screen.dtype != torch.float32 or ft._win is not None or ft._wout is not None:
            return False
        if torch.is_grad_enabled() and (t.requires_grad or screen.requires_grad):
            return False
        n = ft.input_grid.size
        nx = int(ft.input_grid.dims[0])  # the slicing keeps a row of up to 4096 points in registers
        return t.shape[-1] == n and screen.numel() == n and -(-nx // 32) * 32 <= 4096

    def forward_phase_screen(self, e, screen, scale, wavelength=1):
        """``forward`` of the field ``e`` times exp(i scale screen) (a pure phase element such as an atmosphere
        without scintillation ahead of the lens), with the phase applied while the transform slices its input:
        split precision, complex64 fields, uniformly weighted grids; None when the propagator cannot do that here
        (the caller then applies the phase and calls ``forward``)."""
        t = as_tensor(e)
        s = as_tensor(screen)
        if not self.phase_screen_fusable(t, s, wavelength):
            return None
        inst = self.get_instance_data(self._input_grid, None, wavelength)
        ft = inst.fourier_transform
        t = t.contiguous()
        lead = tuple(t.shape[:-1])
        batch = int(np.prod(lead)) if lead else 1
        out = torch.empty(lead + (ft.output_grid.size,), dtype=torch.complex128, device=t.device)
        if batch > 0:
            alpha = complex(ft._w_in_scalar) * inst.norm_factor
            ft._plan(t.dtype).execute_phase(batch, t, s.contiguous(), scale, out, alpha)
        return out

    @make_agnostic_forward
    def forward(self, instance_data, wavefront):
        """fraunhofer.py:56-71: FT.forward(E) * norm_factor (the norm is fused into the GEMM alpha)."""
        ft = instance_data.fourier_transform
        e = wavefront.electric_field
        if isinstance(ft, MatrixFourierTransform):
            alpha = complex(ft._w_in_scalar) * instance_data.norm_factor
            if _differentiable(e):
                from .autograd import mft_apply
                return wavefront._carry(Field(mft_apply(ft, e.data, _lib.HX_FORWARD, alpha), instance_data.output_grid))
            res = ft._run(e, ft.input_grid, ft.output_grid, _lib.HX_FORWARD, alpha)
        else:
            norm = instance_data.norm_factor
            if _differentiable(e):
                from .autograd import linear_apply
                adj = _adjoint_of_forward(ft)
                res = linear_apply(e.data, lambda t: ft.forward(t).data * norm,
                                   lambda g: adj(g) * np.conj(norm))
                return wavefront._carry(Field(res, instance_data.output_grid))
            res = ft.forward(e) * norm
        return wavefront._carry(Field(res.data, instance_data.output_grid))

    @make_agnostic_backward
    def backward(self, instance_data, wavefront):
        """fraunhofer.py:73-88: FT.backward(E) / norm_factor."""
        ft = instance_data.fourier_transform
        e = wavefront.electric_field
        if isinstance(ft, MatrixFourierTransform):
            alpha = complex(ft._w_out_scalar / (2 * np.pi)**ft.ndim) / instance_data.norm_factor
            if _differentiable(e):
                from .autograd import mft_apply
                return wavefront._carry(Field(mft_apply(ft, e.data, _lib.HX_BACKWARD, alpha), instance_data.input_grid))
            res = ft._run(e, ft.output_grid, ft.input_grid, _lib.HX_BACKWARD, alpha)
        else:
            norm = instance_data.norm_factor
            if _differentiable(e):
                from .autograd import linear_apply
                fwd_scale = _adjoint_scale(ft)
                # backward = forward^H / c, so its adjoint is forward / c
                res = linear_apply(e.data, lambda t: ft.backward(t).data / norm,
                                   lambda g: ft.forward(g).data / (fwd_scale * np.conj(norm)))
                return wavefront._carry(Field(res, instance_data.input_grid))
            res = ft.backward(e) / norm
        return wavefront._carry(Field(res.data, instance_data.input_grid))


class AngularSpectrumPropagator(AgnosticOpticalElement):
    """Scalar angular-spectrum propagation over ``distance`` (hcipy/propagation/angular_spectrum.py:7-152).

    The transfer function is built on the device in float64 (native branch,
    :159-166, or the FFT of the impulse response, :143-157), supersampled
    ``num_oversampling`` times, and applied by a Fourier filter with q=2 whose
    multiply is fused into the column FFT pass.
    """

    def __init__(self, input_grid, distance, num_oversampling=2, refractive_index=1):
        self._distance = distance
        self._num_oversampling = num_oversampling
        self._refractive_index = refractive_index
        AgnosticOpticalElement.__init__(self, grid_dependent=True, wavelength_dependent=True)

    def make_instance(self, instance_data, input_grid, output_grid, wavelength):
        import torch
        from .fft import FourierFilter, FastFourierTransform
        from .fourier import make_fft_grid, _is_cartesian
        if not input_grid.is_regular or not _is_cartesian(input_grid):
            raise ValueError('The input grid must be a regular, Cartesian grid.')
        n = self.evaluate_parameter(self.refractive_index, input_grid, output_grid, wavelength)
        k = 2 * np.pi / wavelength * n
        delta = np.asarray(input_grid.delta, np.float64)
        dims = np.asarray(input_grid.dims)
        l_max = np.max(dims * delta)
        os_ = int(round(self.num_oversampling))
        fourier_grid = make_fft_grid(input_grid, 2, 1)
        fz = np.asarray(fourier_grid.zero, np.float64)
        fd = np.asarray(fourier_grid.delta, np.float64)
        fn = [int(d) for d in fourier_grid.dims]
        lib = _lib.lib()
        if np.any(delta < wavelength * abs(self.distance) / l_max):
            # Impulse-response branch: FFT of the supersampled impulse response on the enlarged grid.
            enlarged = make_fft_grid(fourier_grid)
            ez = np.asarray(enlarged.zero, np.float64)
            ed = np.asarray(enlarged.delta, np.float64)
            en = [int(d) for d in enlarged.dims]
            ir = torch.empty(en[0] * en[1], dtype=torch.complex128, device='cuda')
            rc = lib.hx_asp_impulse_response(en[0], en[1], ez[0], ez[1], ed[0], ed[1], k, float(self.distance), os_,
                                             _lib.HX_C128, _lib.dptr(ir), _lib.stream_handle())
            _lib.check(rc, 'hx_asp_impulse_response')
            tf = FastFourierTransform(enlarged).forward(ir).data
            instance_data.fourier_filter = FourierFilter(input_grid, tf, q=2)
        else:
            tf = torch.empty(fn[0] * fn[1], dtype=torch.complex128, device='cuda')
            rc = lib.hx_asp_transfer_function(fn[0], fn[1], fz[0], fz[1], fd[0], fd[1], k, float(self.distance), os_,
                                              _lib.HX_C128, _lib.dptr(tf), _lib.stream_handle())
            _lib.check(rc, 'hx_asp_transfer_function')
            instance_data.fourier_filter = FourierFilter(input_grid, tf, q=2, fft_order=True)

    @property
    def distance(self):
        return self._distance

    @distance.setter
    def distance(self, distance):
        self._distance = distance
        self.clear_cache()

    @property
    def num_oversampling(self):
        return self._num_oversampling

    @num_oversampling.setter
    def num_oversampling(self, num_oversampling):
        self._num_oversampling = num_oversampling
        self.clear_cache()

    @property
    def refractive_index(self):
        return self._refractive_index

    @refractive_index.setter
    def refractive_index(self, refractive_index):
        self._refractive_index = refractive_index
        self.clear_cache()

    def get_input_grid(self, output_grid, wavelength):
        return output_grid

    def get_output_grid(self, input_grid, wavelength):
        return input_grid

    @make_agnostic_forward
    def forward(self, instance_data, wavefront):
        """angular_spectrum.py:206-222; differentiable (the adjoint of the filter is its backward)."""
        return _filter_apply(instance_data.fourier_filter, wavefront, adjoint=False)

    @make_agnostic_backward
    def backward(self, instance_data, wavefront):
        """angular_spectrum.py:224-240; differentiable."""
        return _filter_apply(instance_data.fourier_filter, wavefront, adjoint=True)


class FresnelPropagator(AgnosticOpticalElement):
    """Monochromatic Fresnel propagation over ``distance`` (hcipy/propagation/fresnel.py:8-164).

    The paraxial transfer function exp(i k d) exp(-i d/(2k) (kx^2 + ky^2)) (native branch, :69-80), or the FFT of
    the impulse response exp(i k d)/(i lambda d) exp(i k/(2d) r^2) when the grid undersamples it (:51-67), is
    built on the device in float64, supersampled ``num_oversampling`` times, and applied by a Fourier filter with
    ``q = zero_padding``.  The input grid is taken from the incoming wavefront.
    """

    def __init__(self, input_grid, distance, num_oversampling=2, zero_padding=2, refractive_index=1):
        self._distance = distance
        self._num_oversampling = num_oversampling
        self._zero_padding = zero_padding
        self._refractive_index = refractive_index
        AgnosticOpticalElement.__init__(self, grid_dependent=True, wavelength_dependent=True)

    def make_instance(self, instance_data, input_grid, output_grid, wavelength):
        import torch
        from .fft import FourierFilter, FastFourierTransform
        from .fourier import make_fft_grid, _is_cartesian
        if not input_grid.is_regular or not _is_cartesian(input_grid):
            raise ValueError('The input grid must be a regular, Cartesian grid.')
        n = self.evaluate_parameter(self.refractive_index, input_grid, output_grid, wavelength)
        k = 2 * np.pi / wavelength * n
        delta = np.asarray(input_grid.delta, np.float64)
        l_max = np.max(np.asarray(input_grid.dims) * delta)
        os_ = int(round(self.num_oversampling))
        q = self.zero_padding
        fourier_grid = make_fft_grid(input_grid, q, 1)
        lib = _lib.lib()
        if np.any(delta < wavelength * abs(self.distance) / l_max):
            enlarged = make_fft_grid(fourier_grid)
            ez = np.asarray(enlarged.zero, np.float64)
            ed = np.asarray(enlarged.delta, np.float64)
            en = [int(d) for d in enlarged.dims]
            ir = torch.empty(en[0] * en[1], dtype=torch.complex128, device='cuda')
            rc = lib.hx_fresnel_impulse_response(en[0], en[1], ez[0], ez[1], ed[0], ed[1], k, float(wavelength),
                                                 float(self.distance), os_, _lib.HX_C128, _lib.dptr(ir),
                                                 _lib.stream_handle())
            _lib.check(rc, 'hx_fresnel_impulse_response')
            tf = FastFourierTransform(enlarged).forward(ir).data
            instance_data.fourier_filter = FourierFilter(input_grid, tf, q=q)
        else:
            fz = np.asarray(fourier_grid.zero, np.float64)
            fd = np.asarray(fourier_grid.delta, np.float64)
            fn = [int(d) for d in fourier_grid.dims]
            tf = torch.empty(fn[0] * fn[1], dtype=torch.complex128, device='cuda')
            rc = lib.hx_fresnel_transfer_function(fn[0], fn[1], fz[0], fz[1], fd[0], fd[1], k, float(self.distance),
                                                  os_, _lib.HX_C128, _lib.dptr(tf), _lib.stream_handle())
            _lib.check(rc, 'hx_fresnel_transfer_function')
            instance_data.fourier_filter = FourierFilter(input_grid, tf, q=q, fft_order=True)

    @property
    def distance(self):
        return self._distance

    @distance.setter
    def distance(self, distance):
        self._distance = distance
        self.clear_cache()

    @property
    def num_oversampling(self):
        return self._num_oversampling

    @num_oversampling.setter
    def num_oversampling(self, num_oversampling):
        self._num_oversampling = num_oversampling
        self.clear_cache()

    @property
    def zero_padding(self):
        return self._zero_padding

    @zero_padding.setter
    def zero_padding(self, zero_padding):
        self._zero_padding = zero_padding
        self.clear_cache()

    @property
    def refractive_index(self):
        return self._refractive_index

    @refractive_index.setter
    def refractive_index(self, refractive_index):
        self._refractive_index = refractive_index
        self.clear_cache()

    def get_input_grid(self, output_grid, wavelength):
        return output_grid

    def get_output_grid(self, input_grid, wavelength):
        return input_grid

    @make_agnostic_forward
    def forward(self, instance_data, wavefront):
        """fresnel.py:131-147; differentiable (the adjoint of the filter is its backward)."""
        return _filter_apply(instance_data.fourier_filter, wavefront, adjoint=False)

    @make_agnostic_backward
    def backward(self, instance_data, wavefront):
        """fresnel.py:149-164; differentiable."""
        return _filter_apply(instance_data.fourier_filter, wavefront, adjoint=True)
