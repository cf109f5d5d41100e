"""Wavefronts and optical elements on the device (hcipy/optics).

``Wavefront`` mirrors hcipy/optics/wavefront.py:15-361 for scalar and
partially polarised fields: the electric field is cast to complex of the input
bit depth, ``copy`` is a device copy, the Stokes parameters, ``power`` and
``total_power`` are computed on the GPU.  ``AgnosticOpticalElement`` keeps the reference's instance cache
(hcipy/optics/optical_element.py:261-790): instances keyed by input grid,
output grid and a logarithmic wavelength key, at most 11, first in first out.
"""
import collections
import itertools
import math

import numpy as np
import torch

from .field import Field, as_tensor, grid_key


def jones_stokes(jones, stokes, rows=(0, 1, 2, 3)):
    """Stokes parameters (I, Q, U, V; the ``rows`` asked for) of light with Stokes vector ``stokes`` after the
    Jones matrices ``jones`` (a (2, 2, n) complex tensor): 1/2 M s with M the Mueller matrix of J = [[x, y], [z, w]]
    at every point, written with the products x y*, z w*, ... of its entries (wavefront.py:103-235)."""
    x, y, z, w = jones[0, 0], jones[0, 1], jones[1, 0], jones[1, 1]
    ax, ay, az, aw = (t.real * t.real + t.imag * t.imag for t in (x, y, z, w))
    s = [float(v) for v in stokes]
    out = []
    for k in rows:
        if k == 0:
            xy, zw = x * y.conj(), z * w.conj()
            m = (ax + ay + az + aw, ax - ay + az - aw, 2 * (xy + zw).real, 2 * (xy + zw).imag)
        elif k == 1:
            xy, zw = x * y.conj(), z * w.conj()
            m = (ax + ay - az - aw, ax - ay - az + aw, 2 * (xy - zw).real, 2 * (xy - zw).imag)
        elif k == 2:
            xz, yw, xw, yz = x * z.conj(), y * w.conj(), x * w.conj(), y * z.conj()
            m = (2 * (xz + yw).real, 2 * (xz - yw).real, 2 * (xw + yz).real, 2 * (xw - yz).imag)
        else:
            xz, yw, xw, yz = x * z.conj(), y * w.conj(), x * w.conj(), y * z.conj()
            m = (-2 * (xz + yw).imag, -2 * (xz - yw).imag, -2 * (xw + yz).imag, 2 * (xw - yz).real)
        out.append(0.5 * (m[0] * s[0] + m[1] * s[1] + m[2] * s[2] + m[3] * s[3]))
    return out


class Wavefront(object):
    """A wavefront: a device Field of the electric field and a wavelength (hcipy/optics/wavefront.py).

    Leading axes of the field are a batch of scalar fields.  With ``input_stokes_vector`` (I, Q, U, V) the wavefront
    is partially polarised (wavefront.py:47-66): its field is the 2x2 Jones matrix of the system at every point,
    shape (2, 2, n), which a scalar field becomes as E times the identity; the Stokes parameters of the light are
    then the Mueller matrix of that Jones matrix applied to the input Stokes vector.
    """

    def __init__(self, electric_field, wavelength=1, input_stokes_vector=None):
        stokes = None
        if input_stokes_vector is not None:
            if not hasattr(electric_field, 'grid'):
                raise ValueError('The electric field must be a Field.')
            t = as_tensor(electric_field)
            if t.dim() == 1:
                z = torch.zeros_like(t)
                t = torch.stack((torch.stack((t, z)), torch.stack((z, t))))
            elif tuple(t.shape[:-1]) != (2, 2):
                raise ValueError('When supplying a Stokes vector, the electric field must be either a scalar or '
                                 '2-tensor field.')
            electric_field = Field(t, electric_field.grid)
            stokes = np.array(input_stokes_vector, dtype=np.float64)
            if stokes.shape != (4,):
                raise ValueError('A Stokes vector has four components (I, Q, U, V).')
        self.electric_field = electric_field
        self.wavelength = wavelength
        self._input_stokes_vector = stokes

    @property
    def electric_field(self):
        return self._electric_field

    @electric_field.setter
    def electric_field(self, field):
        # hcipy/optics/wavefront.py:77-88: complex of the same bit depth.
        if not hasattr(field, 'grid'):
            raise ValueError('The electric field must be a Field.')
        grid = field.grid
        t = as_tensor(field)
        dt = torch.complex64 if t.dtype in (torch.float32, torch.complex64) else torch.complex128
        if t.dtype != dt:
            t = t.to(dt)
        self._electric_field = Field(t, grid)

    @property
    def input_stokes_vector(self):
        """The Stokes vector of the light that the Jones matrices act on (None for a scalar wavefront)."""
        return self._input_stokes_vector

    @property
    def is_polarized(self):
        return self._input_stokes_vector is not None

    is_partially_polarized = is_polarized

    @property
    def is_scalar(self):
        return self._input_stokes_vector is None

    @property
    def wavenumber(self):
        return 2 * np.pi / self.wavelength

    @property
    def grid(self):
        return self._electric_field.grid

    def copy(self):
        return Wavefront(self._electric_field.copy(), self.wavelength, self._input_stokes_vector)

    def _carry(self, field):
        """A wavefront of ``field`` with this wavefront's wavelength and input Stokes vector."""
        return Wavefront(field, self.wavelength, self._input_stokes_vector)

    @property
    def I(self):  # noqa: N802
        if self.is_polarized:
            return Field(jones_stokes(self._electric_field.data, self._input_stokes_vector, (0,))[0], self.grid)
        e = self._electric_field.data
        return Field(e.real * e.real + e.imag * e.imag, self.grid)

    intensity = I

    def _stokes_part(self, k):
        if self.is_polarized:
            return Field(jones_stokes(self._electric_field.data, self._input_stokes_vector, (k,))[0], self.grid)
        e = self._electric_field.data
        return Field(torch.zeros(e.shape, dtype=e.real.dtype, device=e.device), self.grid)

    @property
    def Q(self):  # noqa: N802
        return self._stokes_part(1)

    @property
    def U(self):  # noqa: N802
        return self._stokes_part(2)

    @property
    def V(self):  # noqa: N802
        return self._stokes_part(3)

    @property
    def stokes_vector(self):
        """(4, n): I, Q, U, V (a scalar wavefront is unpolarised: I = |E|^2, the rest 0)."""
        if self.is_polarized:
            return Field(torch.stack(jones_stokes(self._electric_field.data, self._input_stokes_vector)), self.grid)
        i = self.I.data
        out = torch.zeros(tuple(i.shape[:-1]) + (4, i.shape[-1]), dtype=i.dtype, device=i.device)
        out[..., 0, :] = i
        return Field(out, self.grid)

    @property
    def degree_of_polarization(self):
        i, q, u, v = self.I.data, self.Q.data, self.U.data, self.V.data
        return Field(torch.sqrt(q**2 + u**2 + v**2) / i, self.grid)

    @property
    def degree_of_linear_polarization(self):
        i, q, u = self.I.data, self.Q.data, self.U.data
        return Field(torch.sqrt(q**2 + u**2) / i, self.grid)

    @property
    def angle_of_linear_polarization(self):
        return Field(0.5 * torch.atan2(self.U.data, self.Q.data), self.grid)

    @property
    def degree_of_circular_polarization(self):
        return Field(self.V.data / self.I.data, self.grid)

    @property
    def ellipticity(self):
        i, q, u, v = self.I.data, self.Q.data, self.U.data, self.V.data
        return Field(v / (i + torch.sqrt(q**2 + u**2)), self.grid)

    @property
    def amplitude(self):
        return Field(self._electric_field.data.abs(), self.grid)

    @property
    def phase(self):
        return Field(torch.angle(self._electric_field.data), self.grid)

    @property
    def power(self):
        w = self.grid.weights
        w = torch.as_tensor(w, device=self._electric_field.data.device) if not np.isscalar(w) else w
        return Field(self.I.data * w, self.grid)

    @property
    def total_power(self):
        return self.power.data.sum(-1)


class OpticalElement(object):
    """Base class: forward/backward map a Wavefront to a Wavefront (hcipy/optics/optical_element.py:6-151)."""

    def __call__(self, wavefront):
        return self.forward(wavefront)

    def forward(self, wavefront):
        raise NotImplementedError()

    def backward(self, wavefront):
        raise NotImplementedError()


class EmptyOpticalElement(OpticalElement):
    """An element that leaves the wavefront unchanged, to stand in for an optional element
    (hcipy/optics/optical_element.py:153-218)."""

    def forward(self, wavefront):
        return wavefront

    def backward(self, wavefront):
        return wavefront


class OpticalSystem(OpticalElement):
    """A linear path of optical elements (hcipy/optics/optical_element.py:848-950): ``forward`` applies them in
    order, ``backward`` applies their backward propagations in reverse order."""

    def __init__(self, optical_elements):
        self.optical_elements = optical_elements

    @property
    def optical_elements(self):
        return self._optical_elements

    @optical_elements.setter
    def optical_elements(self, optical_elements):
        self._optical_elements = list(optical_elements)

    def forward(self, wavefront):
        wf = wavefront
        for element in self._optical_elements:
            wf = element.forward(wf)
        return wf

    def backward(self, wavefront):
        wf = wavefront
        for element in reversed(self._optical_elements):
            wf = element.backward(wf)
        return wf


class InstanceData(object):
    def __init__(self, input_grid, output_grid, wavelength):
        self.input_grid = input_grid
        self.output_grid = output_grid
        self.wavelength = wavelength


def _wavelength_key(wavelength):
    # hcipy/optics/optical_element.py:333.
    return int(np.round(np.log(wavelength) / np.log(1 + 1e-9)))


class AgnosticOpticalElement(OpticalElement):
    """Optical element whose device state depends on the grids and the wavelength it is used with."""

    def __init__(self, grid_dependent=True, wavelength_dependent=True, max_in_cache=11):
        self._grid_dependent = grid_dependent
        self._wavelength_dependent = wavelength_dependent
        self._max_in_cache = max_in_cache
        self.clear_cache()

    def clear_cache(self):
        self._cache = collections.OrderedDict()
        self._instances = collections.OrderedDict()

    def _keys(self, input_grid, output_grid, wavelength):
        grid_parts = [(None, None)]
        if self._grid_dependent:
            ki = None if input_grid is None else grid_key(input_grid)
            ko = None if output_grid is None else grid_key(output_grid)
            if ki is None and ko is None:
                raise ValueError('Grid dependent, but no grids are given for lookup.')
            if ki is None or ko is None:
                grid_parts = [(ki, ko)]
            else:
                grid_parts = [(ki, ko), (ki, None), (None, ko)]
        wl_part = (None,)
        if self._wavelength_dependent:
            if wavelength is None:
                raise ValueError('Wavelength dependent, but no wavelength is given for lookup.')
            wl_part = (_wavelength_key(wavelength),)
        return [g + wl_part for g in grid_parts]

    def get_instance_data(self, input_grid, output_grid, wavelength):
        for key in self._keys(input_grid, output_grid, wavelength):
            if key in self._cache:
                return self._cache[key]
        if input_grid is None:
            input_grid = self.get_input_grid(output_grid, wavelength)
        if output_grid is None:
            output_grid = self.get_output_grid(input_grid, wavelength)
        keys = self._keys(input_grid, output_grid, wavelength)
        for key in keys:
            if key in self._cache:
                return self._cache[key]
        inst = InstanceData(input_grid, output_grid, wavelength)
        self.make_instance(inst, input_grid, output_grid, wavelength)
        if len(self._instances) >= self._max_in_cache:
            _, (old, old_keys) = self._instances.popitem(last=False)
            for k in old_keys:
                self._cache.pop(k, None)
        self._instances[id(inst)] = (inst, keys)
        for key in keys:
            self._cache[key] = inst
        return inst

    def make_instance(self, instance_data, input_grid, output_grid, wavelength):
        pass

    def get_input_grid(self, output_grid, wavelength):
        raise ValueError('This optical element cannot infer its input grid.')

    def get_output_grid(self, input_grid, wavelength):
        raise ValueError('This optical element cannot infer its output grid.')

    def evaluate_parameter(self, parameter, input_grid, output_grid, wavelength):
        if callable(parameter):
            return parameter(wavelength)
        return parameter


def make_agnostic_forward(forward):
    def res(self, wavefront, *args, **kwargs):
        inst = self.get_instance_data(wavefront.grid, None, wavefront.wavelength)
        return forward(self, inst, wavefront, *args, **kwargs)
    return res


def make_agnostic_backward(backward):
    def res(self, wavefront, *args, **kwargs):
        inst = self.get_instance_data(None, wavefront.grid, wavefront.wavelength)
        return backward(self, inst, wavefront, *args, **kwargs)
    return res


def _apodization_tensor(a, wavelength, like):
    if callable(a):
        a = a(wavelength)
    if np.isscalar(a):
        return a
    return as_tensor(a, like.device)


class Apodizer(OpticalElement):
    """A thin apodizer: E * a forward, E * conj(a) backward (hcipy/optics/apodization.py:6-35)."""

    def __init__(self, apodization):
        self.apodization = apodization

    def forward(self, wavefront):
        e = wavefront.electric_field
        a = _apodization_tensor(self.apodization, wavefront.wavelength, e.data)
        return wavefront._carry(Field(e.data * a, e.grid))

    def backward(self, wavefront):
        e = wavefront.electric_field
        a = _apodization_tensor(self.apodization, wavefront.wavelength, e.data)
        a = a.conj() if isinstance(a, torch.Tensor) else np.conj(a)
        return wavefront._carry(Field(e.data * a, e.grid))


class PhaseApodizer(OpticalElement):
    """E * exp(+-i phase) (hcipy/optics/apodization.py:37-62)."""

    def __init__(self, phase):
        self._phase = phase

    @property
    def phase(self):
        return self._phase

    def _apply(self, wavefront, sign):
        from .kernels import apply_phase
        e = wavefront.electric_field
        if np.isscalar(self._phase) or np.ndim(self._phase) == 0:  # a uniform phase, as the reference allows
            phase = torch.full((e.data.shape[-1],), float(np.asarray(self._phase)), dtype=torch.float64,
                               device=e.data.device)
        else:
            phase = as_tensor(self._phase, e.data.device)
        return wavefront._carry(Field(apply_phase(e.data, phase, sign), e.grid))

    def forward(self, wavefront):
        return self._apply(wavefront, 1.0)

    def backward(self, wavefront):
        return self._apply(wavefront, -1.0)


class SurfaceApodizer(OpticalElement):
    """A thin transmissive plate of sag ``surface_sag``: E * exp(+-i (n - 1) sag 2 pi / lambda), n the refractive
    index (a scalar or a function of the wavelength) (hcipy/optics/apodization.py:64-102)."""

    def __init__(self, surface_sag, refractive_index):
        self.surface_sag = surface_sag
        self.refractive_index = refractive_index

    def _get_refractive_index(self, wavelength):
        return self.refractive_index(wavelength) if callable(self.refractive_index) else self.refractive_index

    def _apply(self, wavefront, sign):
        from .kernels import apply_phase
        e = wavefront.electric_field
        scale = sign * (self._get_refractive_index(wavefront.wavelength) - 1) * 2 * np.pi / wavefront.wavelength
        sag = as_tensor(self.surface_sag, e.data.device)
        return wavefront._carry(Field(apply_phase(e.data, sag, scale), e.grid))

    def forward(self, wavefront):
        return self._apply(wavefront, 1.0)

    def backward(self, wavefront):
        return self._apply(wavefront, -1.0)
