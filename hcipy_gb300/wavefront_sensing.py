"""Pyramid wavefront-sensor optics (hcipy/wavefront_sensing/pyramid.py:94-199) on the Fourier operators.

The sensor is a lens to a focal plane, a circular field stop times the phase of a glass pyramid, and a second lens
to the sensor's pupil plane.  When the first lens is a matrix Fourier transform, the stop and the pyramid phase
(one complex mask per wavelength, built once on the device) are the epilogue of its last GEMM, so a propagation
is two transforms.
"""
import math

import numpy as np
import torch

from . import _lib
from .field import Field, as_tensor, make_pupil_grid
from .fourier import MatrixFourierTransform
from .optics import OpticalElement, Wavefront
from .propagation import FraunhoferPropagator
from .workloads import circular_aperture


class PyramidWavefrontSensorOptics(OpticalElement):
    """The optics of a pyramid wavefront sensor (pyramid.py:94-199), same arguments and defaults."""

    def __init__(self, input_grid, output_grid, separation=None, pupil_diameter=None, wavelength_0=1, q=None,
                 num_airy=None, refractive_index=lambda x: 1.5):
        if not input_grid.is_regular:
            raise ValueError('The input grid must be a regular grid.')
        self.input_grid = input_grid
        self.output_grid = output_grid
        d_in = np.asarray(input_grid.delta, np.float64) * np.asarray(input_grid.dims)
        d_out = np.asarray(output_grid.delta, np.float64) * np.asarray(output_grid.dims)
        if pupil_diameter is None:
            pupil_diameter = float(np.max(d_in))
        if separation is None:
            separation = pupil_diameter
        # pyramid.py:129-135: at least 2 pixels per resolution element, and enough to sample the output plane
        qmin = math.ceil(max(float(np.max(d_out / d_in)), 2))
        if q is None:
            q = qmin
        elif q < qmin:
            raise ValueError('The requested focal plane sampling is too low to sufficiently sample the wavefront '
                             'sensor output.')
        self.num_airy = float(np.max(input_grid.shape)) / 2 if num_airy is None else num_airy
        num_pixels = 2 * int(self.num_airy * q)
        spatial_resolution = wavelength_0 / pupil_diameter
        self.focal_grid = make_pupil_grid(num_pixels, 2 * spatial_resolution * self.num_airy)
        self._separation = separation
        self._refractive_index = refractive_index
        self._wavelength_0 = wavelength_0
        self._stop = circular_aperture(self.focal_grid, 2 * self.num_airy * wavelength_0 / pupil_diameter)
        x, y = self.focal_grid.points_list()
        self._surface = -separation / (2 * (refractive_index(wavelength_0) - 1)) * (np.abs(x) + np.abs(y))
        self.pupil_to_focal = FraunhoferPropagator(input_grid, self.focal_grid)
        self.focal_to_pupil = FraunhoferPropagator(self.focal_grid, output_grid)
        self._masks = {}

    def _mask(self, wavelength, dtype, conj):
        """stop * exp(+-i (n(lambda) - 1) surface 2 pi / lambda) on the focal grid (pyramid.py:148-151 with
        SurfaceApodizer, apodization.py:88-102)."""
        key = (float(wavelength), dtype, conj)
        m = self._masks.get(key)
        if m is None:
            n = self._refractive_index(wavelength)
            phase = (n - 1) * self._surface * 2 * np.pi / wavelength
            m = self._stop * np.exp((-1j if conj else 1j) * phase)
            m = torch.from_numpy(m.astype(np.complex64 if dtype == torch.complex64 else np.complex128)).cuda()
            self._masks[key] = m
        return m

    def _to_focal(self, wavefront, conj):
        """Lens, stop and pyramid (or their adjoint order for conj): the mask fused into the MFT's epilogue."""
        e = as_tensor(wavefront.electric_field).contiguous()
        wl = wavefront.wavelength
        inst = self.pupil_to_focal.get_instance_data(self.input_grid, self.focal_grid, wl)
        ft = inst.fourier_transform
        mask = self._mask(wl, e.dtype, conj)
        if isinstance(ft, MatrixFourierTransform) and not conj:
            alpha = complex(ft._w_in_scalar) * inst.norm_factor
            focal = ft._run(e, ft.input_grid, ft.output_grid, _lib.HX_FORWARD, alpha, epilogue=_lib.HX_EPI_MUL,
                            mask=mask).data
        else:
            focal = self.pupil_to_focal.forward(wavefront).electric_field.data * mask
        return focal

    def forward(self, wavefront):
        """pyramid.py:164-181."""
        focal = self._to_focal(wavefront, False)
        return self.focal_to_pupil.forward(Wavefront(Field(focal, self.focal_grid), wavefront.wavelength))

    def backward(self, wavefront):
        """pyramid.py:183-199."""
        focal = self.focal_to_pupil.backward(wavefront).electric_field.data
        focal = focal * self._mask(wavefront.wavelength, focal.dtype, True)
        return self.pupil_to_focal.backward(Wavefront(Field(focal, self.focal_grid), wavefront.wavelength))
