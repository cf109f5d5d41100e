"""Pyramid wavefront-sensor optics (hcipy/wavefront_sensing/pyramid.py), plain and modulated, on the Fourier
operators.

The sensor is a lens to a focal plane, a circular field stop times the phase of a glass pyramid, and a second lens
to the sensor's pupil plane.  When the first lens is a matrix Fourier transform, the stop and the pyramid phase
(one complex mask per wavelength, built once on the device) are the epilogue of its last GEMM, so a propagation
is two transforms.  The modulated sensor runs all its modulation steps as one batch of fields.
"""
import math

import numpy as np
import torch

from . import _lib
from .deformable_mirror import TipTiltMirror
from .field import CartesianGrid, Field, UnstructuredCoords, as_tensor, make_pupil_grid
from .fourier import MatrixFourierTransform
from .kernels import apply_phase
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
        self._stops = {}

    def _stop_mask(self, dtype):
        """The field stop alone (the spatial filter, pyramid.py:146) as a device mask."""
        m = self._stops.get(dtype)
        if m is None:
            m = torch.from_numpy(self._stop.astype(np.complex64 if dtype == torch.complex64 else np.complex128)).cuda()
            self._stops[dtype] = m
        return m

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

    def _to_focal(self, wavefront, pyramid=True):
        """The first lens times the stop and (with ``pyramid``) the pyramid phase, the mask fused into the MFT's
        epilogue."""
        e = as_tensor(wavefront.electric_field).contiguous()
        wl = wavefront.wavelength
        inst = self.pupil_to_focal.get_instance_data(self.input_grid, self.focal_grid, wl)
        ft = inst.fourier_transform
        mask = self._mask(wl, e.dtype, False) if pyramid else self._stop_mask(e.dtype)
        if isinstance(ft, MatrixFourierTransform):
            alpha = complex(ft._w_in_scalar) * inst.norm_factor
            focal = ft._run(e, ft.input_grid, ft.output_grid, _lib.HX_FORWARD, alpha, epilogue=_lib.HX_EPI_MUL,
                            mask=mask).data
        else:
            focal = self.pupil_to_focal.forward(wavefront).electric_field.data * mask
        return focal

    def forward(self, wavefront):
        """pyramid.py:164-181."""
        focal = self._to_focal(wavefront)
        return self.focal_to_pupil.forward(Wavefront(Field(focal, self.focal_grid), wavefront.wavelength))

    def backward(self, wavefront):
        """pyramid.py:183-199."""
        focal = self.focal_to_pupil.backward(wavefront).electric_field.data
        focal = focal * self._mask(wavefront.wavelength, focal.dtype, True)
        return self.pupil_to_focal.backward(Wavefront(Field(focal, self.focal_grid), wavefront.wavelength))


def _dithered_deltas(c):
    """Per-point spacing of a separated axis (hcipy/field/util.py:661-665): the central difference inside, the
    one-sided difference at both ends."""
    return np.concatenate(([c[1] - c[0]], (c[2:] - c[:-2]) / 2., [c[-1] - c[-2]]))


class ModulatedPyramidWavefrontSensorOptics(OpticalElement):
    """The optics of a modulated pyramid wavefront sensor (pyramid.py:10-91), same arguments and both methods.

    The modulation steps are one batch of fields.  Tip-tilt method (the default): the tip-tilt mirror reflects the
    input at every modulation position in one phase launch (its surfaces for all positions are one sparse product)
    and the batch goes through the pyramid optics as two batched transforms.  Fast method: the input goes to the
    focal plane once with the field stop fused into the transform, each step's shifted pyramid phase is applied in
    one launch over the batch, and one batched transform returns to the sensor's pupil plane; the shifted pyramid
    surfaces are sampled four times per pixel and axis and averaged, at plan time on the host, as in the reference.

    ``forward`` returns one wavefront per modulation step (views of the batch).  There is no ``backward``: the
    reference refuses it as non-physical.
    """

    def __init__(self, pyramid_wavefront_sensor, modulation, num_steps=12, fast_modulation_method=False):
        self.modulation = modulation
        self.pyramid_wavefront_sensor = pyramid_wavefront_sensor
        self.tip_tilt_mirror = TipTiltMirror(pyramid_wavefront_sensor.input_grid)
        self.focal_grid = pyramid_wavefront_sensor.focal_grid
        self.pupil_to_focal = pyramid_wavefront_sensor.pupil_to_focal
        self.focal_to_pupil = pyramid_wavefront_sensor.focal_to_pupil
        self._fast_modulation_method = fast_modulation_method
        # pyramid.py:39-44: num_steps points on a circle of radius modulation / 2 (the mirror doubles the tilt)
        theta = np.linspace(0, 2 * np.pi, num_steps, endpoint=False)
        self._positions = np.stack((modulation / 2 * np.cos(theta), modulation / 2 * np.sin(theta)), axis=1)
        self.modulation_positions = CartesianGrid(UnstructuredCoords((self._positions[:, 0], self._positions[:, 1])))
        self._sags = self._shifted_pyramid_sags() if fast_modulation_method else None
        self._phases = {}

    def _shifted_pyramid_sags(self, oversampling=4):
        """The pyramid's sag on the focal grid shifted by twice each modulation position (pyramid.py:50-63), each
        pixel the mean of oversampling^2 dithered samples (util.py:651-690)."""
        pwfs = self.pyramid_wavefront_sensor
        c = -pwfs._separation / (2 * (pwfs._refractive_index(pwfs._wavelength_0) - 1))
        dither = (np.arange(oversampling) + 0.5) / oversampling - 0.5
        sags = np.empty((len(self._positions), self.focal_grid.size))
        for k, p in enumerate(self._positions):
            xs, ys = self.focal_grid.shifted(2 * p).separated_coords
            dx, dy = _dithered_deltas(xs), _dithered_deltas(ys)
            acc = 0
            for ty in dither:  # dither points in field order, x fastest
                for tx in dither:
                    ax, ay = np.abs(xs + tx * dx), np.abs(ys + ty * dy)
                    acc = acc + c * (ax[np.newaxis, :] + ay[:, np.newaxis]).ravel()
            sags[k] = acc / oversampling**2
        return sags

    def _fast_phase(self, wavelength, dtype):
        """(n(lambda) - 1) sag 2 pi / lambda of every shifted pyramid (apodization.py:88-93), reduced to
        [-pi, pi] in float64 before the cast so that complex64 keeps the phase's full relative precision."""
        key = (float(wavelength), dtype)
        ph = self._phases.get(key)
        if ph is None:
            n = self.pyramid_wavefront_sensor._refractive_index(wavelength)
            phase = (n - 1) * self._sags * (2 * np.pi / wavelength)
            phase = phase - 2 * np.pi * np.round(phase / (2 * np.pi))
            ph = torch.from_numpy(phase.astype(np.float32 if dtype == torch.complex64 else np.float64)).cuda()
            self._phases[key] = ph
        return ph

    def _modulate_one(self, wavefront):
        """All modulation steps of one field: (num_steps, npix_out)."""
        pwfs = self.pyramid_wavefront_sensor
        wl = wavefront.wavelength
        if self._fast_modulation_method:
            focal = pwfs._to_focal(wavefront, pyramid=False)
            steps = apply_phase(focal, self._fast_phase(wl, focal.dtype), 1.0)
            return self.focal_to_pupil.forward(Wavefront(Field(steps, self.focal_grid), wl)).electric_field.data
        self.tip_tilt_mirror.actuators = torch.from_numpy(self._positions)
        try:
            tilted = self.tip_tilt_mirror.forward(wavefront)
        finally:
            # the reference leaves the mirror at the last modulation position
            self.tip_tilt_mirror.actuators = self._positions[-1].copy()
        return pwfs.forward(tilted).electric_field.data

    def forward(self, wavefront):
        """pyramid.py:65-88: one output wavefront per modulation step.  A wavefront holding a batch of fields
        (..., npix) gives steps of shape (..., npix_out)."""
        e = as_tensor(wavefront.electric_field)
        lead = tuple(e.shape[:-1])
        wl = wavefront.wavelength
        grid = wavefront.electric_field.grid
        if not lead:
            out = self._modulate_one(Wavefront(Field(e, grid), wl))
        else:
            flat = e.reshape((-1, e.shape[-1]))
            out = torch.stack([self._modulate_one(Wavefront(Field(flat[j], grid), wl)) for j in range(flat.shape[0])],
                              dim=1)
            out = out.reshape((out.shape[0],) + lead + (out.shape[-1],))
        return [Wavefront(Field(out[k], self.pyramid_wavefront_sensor.output_grid), wl) for k in range(out.shape[0])]

    def backward(self, wavefront):
        raise RuntimeError('This is a non-physical operation.')
