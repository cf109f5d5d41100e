"""Propagators (hcipy/propagation) on the device."""
import numpy as np

from . import _lib
from .field import Field
from .fourier import make_fourier_transform, MatrixFourierTransform
from .optics import AgnosticOpticalElement, Wavefront, make_agnostic_forward, make_agnostic_backward


class FraunhoferPropagator(AgnosticOpticalElement):
    """A perfect lens from its front to its back focal plane (hcipy/propagation/fraunhofer.py:7-88).

    ``precision`` ('fp32' or 'split') is forwarded to the matrix Fourier
    transform when the planner picks one.
    """

    def __init__(self, input_grid, output_grid, focal_length=1, precision='fp32'):
        self._input_grid = input_grid
        self._output_grid = output_grid
        self._focal_length = focal_length
        self.precision = precision
        AgnosticOpticalElement.__init__(self, grid_dependent=True, wavelength_dependent=True)

    def make_instance(self, instance_data, input_grid, output_grid, wavelength):
        # fraunhofer.py:32-38.
        focal_length = self.evaluate_parameter(self.focal_length, input_grid, output_grid, wavelength)
        instance_data.uv_grid = output_grid.scaled(2 * np.pi / (focal_length * wavelength))
        ft = make_fourier_transform(input_grid, instance_data.uv_grid)
        if isinstance(ft, MatrixFourierTransform) and self.precision != 'fp32':
            ft = MatrixFourierTransform(input_grid, instance_data.uv_grid, precision=self.precision)
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

    @make_agnostic_forward
    def forward(self, instance_data, wavefront):
        """fraunhofer.py:56-71: FT.forward(E) * norm_factor (the norm is fused into the GEMM alpha)."""
        ft = instance_data.fourier_transform
        e = wavefront.electric_field
        if isinstance(ft, MatrixFourierTransform):
            res = ft._run(e, ft.input_grid, ft.output_grid, _lib.HX_FORWARD,
                          complex(ft._w_in_scalar) * instance_data.norm_factor)
        else:
            res = ft.forward(e) * instance_data.norm_factor
        return Wavefront(Field(res.data, instance_data.output_grid), wavefront.wavelength)

    @make_agnostic_backward
    def backward(self, instance_data, wavefront):
        """fraunhofer.py:73-88: FT.backward(E) / norm_factor."""
        ft = instance_data.fourier_transform
        e = wavefront.electric_field
        if isinstance(ft, MatrixFourierTransform):
            alpha = complex(ft._w_out_scalar / (2 * np.pi)**ft.ndim) / instance_data.norm_factor
            res = ft._run(e, ft.output_grid, ft.input_grid, _lib.HX_BACKWARD, alpha)
        else:
            res = ft.backward(e) / instance_data.norm_factor
        return Wavefront(Field(res.data, instance_data.input_grid), wavefront.wavelength)
