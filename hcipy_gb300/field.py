"""Grids and device-backed Fields.

Grids are host objects (coordinates in float64 numpy), mirroring HCIPy's
``CartesianGrid`` with ``RegularCoords`` / ``SeparatedCoords`` /
``UnstructuredCoords`` (hcipy/field/cartesian_grid.py, hcipy/field/coordinates.py)
and its grid factories (hcipy/field/util.py:68-318).

A ``Field`` couples a CUDA ``torch.Tensor`` with its grid, in the style of the
reference's array-API ``NewStyleField`` (hcipy/field/field.py:308-727): the
values live in ``field.data`` (shape ``tensor_shape + (grid.size,)``), element
arithmetic delegates to torch and keeps the grid.  Operators of this package
accept Fields, CUDA tensors, numpy arrays and reference (numpy) Fields, and
return Fields on the device.

Operators also accept the reference's own grid objects: they read only the
attributes both share (``is_regular``, ``is_separated``, ``dims``, ``delta``,
``zero``, ``separated_coords``, ``weights``, ``ndim``, ``size``).
"""
import hashlib
import math
from collections.abc import Iterable

import numpy as np
import torch

# ---------------------------------------------------------------------------
# Coordinates
# ---------------------------------------------------------------------------


class RegularCoords(object):
    """Regularly spaced coordinates: zero + delta * arange(dims) per axis (hcipy/field/coordinates.py:557-640)."""
    is_regular = True
    is_separated = True
    is_unstructured = False

    def __init__(self, delta, dims, zero):
        n = max(np.size(delta), np.size(dims), np.size(zero))
        self.delta = np.broadcast_to(np.asarray(delta, np.float64), (n,)).copy()
        self.dims = np.broadcast_to(np.asarray(dims, np.int64), (n,)).copy()
        self.zero = np.broadcast_to(np.asarray(zero, np.float64), (n,)).copy()

    @property
    def ndim(self):
        return len(self.dims)

    @property
    def size(self):
        return int(np.prod(self.dims))

    @property
    def separated_coords(self):
        return [self.zero[i] + self.delta[i] * np.arange(self.dims[i]) for i in range(self.ndim)]

    def scaled(self, s):
        s = np.broadcast_to(np.asarray(s, np.float64), (self.ndim,))
        return RegularCoords(self.delta * s, self.dims, self.zero * s)

    def shifted(self, s):
        return RegularCoords(self.delta, self.dims, self.zero + np.asarray(s, np.float64))

    def key(self):
        return ('regular', self.delta.tobytes(), self.dims.tobytes(), self.zero.tobytes())


class SeparatedCoords(object):
    """A tensor product of arbitrary 1-D coordinate arrays (hcipy/field/coordinates.py:420-555)."""
    is_regular = False
    is_separated = True
    is_unstructured = False

    def __init__(self, separated_coords):
        self._coords = [np.asarray(c, np.float64).copy() for c in separated_coords]

    @property
    def separated_coords(self):
        return [c.copy() for c in self._coords]

    @property
    def dims(self):
        return np.array([len(c) for c in self._coords], np.int64)

    @property
    def ndim(self):
        return len(self._coords)

    @property
    def size(self):
        return int(np.prod(self.dims))

    def scaled(self, s):
        s = np.broadcast_to(np.asarray(s, np.float64), (self.ndim,))
        return SeparatedCoords([c * si for c, si in zip(self._coords, s)])

    def shifted(self, s):
        s = np.broadcast_to(np.asarray(s, np.float64), (self.ndim,))
        return SeparatedCoords([c + si for c, si in zip(self._coords, s)])

    def key(self):
        return ('separated',) + tuple(c.tobytes() for c in self._coords)


class UnstructuredCoords(object):
    """Arbitrary point lists; the Fourier operators of this package reject them."""
    is_regular = False
    is_separated = False
    is_unstructured = True

    def __init__(self, coords):
        self._coords = [np.asarray(c, np.float64).copy() for c in coords]

    @property
    def ndim(self):
        return len(self._coords)

    @property
    def size(self):
        return len(self._coords[0])

    @property
    def dims(self):
        raise ValueError('An unstructured grid has no dims.')

    def scaled(self, s):
        s = np.broadcast_to(np.asarray(s, np.float64), (self.ndim,))
        return UnstructuredCoords([c * si for c, si in zip(self._coords, s)])

    def shifted(self, s):
        s = np.broadcast_to(np.asarray(s, np.float64), (self.ndim,))
        return UnstructuredCoords([c + si for c, si in zip(self._coords, s)])

    def key(self):
        return ('unstructured',) + tuple(c.tobytes() for c in self._coords)

    def flat(self):
        return [c.copy() for c in self._coords]


# ---------------------------------------------------------------------------
# Cartesian grid
# ---------------------------------------------------------------------------


class CartesianGrid(object):
    """A Cartesian grid (hcipy/field/cartesian_grid.py).  Flat order is x fastest (shape = dims reversed)."""

    def __init__(self, coords, weights=None):
        self.coords = coords
        self._weights = weights

    # -- structure --------------------------------------------------------
    def is_(self, system):
        return system == 'cartesian'

    def as_(self, system):
        if system != 'cartesian':
            raise ValueError('Only Cartesian grids are supported by hcipy_gb300.')
        return self

    @property
    def is_regular(self):
        return self.coords.is_regular

    @property
    def is_separated(self):
        return self.coords.is_separated

    @property
    def is_unstructured(self):
        return self.coords.is_unstructured

    @property
    def ndim(self):
        return self.coords.ndim

    @property
    def size(self):
        return self.coords.size

    @property
    def dims(self):
        return self.coords.dims

    @property
    def shape(self):
        return tuple(int(d) for d in self.dims[::-1])

    @property
    def delta(self):
        if not self.is_regular:
            raise ValueError('A non-regular grid has no delta.')
        return self.coords.delta

    @property
    def zero(self):
        if not self.is_regular:
            raise ValueError('A non-regular grid has no zero.')
        return self.coords.zero

    @property
    def separated_coords(self):
        return self.coords.separated_coords

    def points_list(self):
        """Flat coordinate arrays (one per axis) in field order."""
        if self.is_separated:
            axes = self.separated_coords
            if self.ndim == 1:
                return [axes[0]]
            mesh = np.meshgrid(*axes[::-1], indexing='ij')[::-1]
            return [m.ravel() for m in mesh]
        return self.coords.flat()

    @property
    def x(self):
        return self.points_list()[0]

    @property
    def y(self):
        return self.points_list()[1]

    @property
    def points(self):
        return np.stack(self.points_list(), axis=-1)

    # -- weights (hcipy/field/cartesian_grid.py:167-189) -------------------
    @property
    def weights(self):
        if self._weights is not None:
            return self._weights
        if self.is_regular:
            return float(np.prod(self.delta))
        if self.is_separated:
            w = None
            for i, x in enumerate(self.separated_coords):
                wi = np.concatenate(([x[1] - x[0]], (x[2:] - x[:-2]) / 2, [x[-1] - x[-2]])) if len(x) > 1 else np.ones(1)
                shape = (1,) * (self.ndim - i - 1) + (-1,) + (1,) * i
                wi = wi.reshape(shape)
                w = wi if w is None else w * wi
            return w.ravel()
        raise ValueError('Weights of an unstructured grid must be given explicitly.')

    @weights.setter
    def weights(self, w):
        self._weights = w

    def separated_weights(self):
        """Per-axis weights (list of arrays) of a separated grid, or None when the weight is a scalar."""
        if self.is_regular and self._weights is None:
            return None
        w_axes = []
        for x in self.separated_coords:
            if len(x) > 1:
                w_axes.append(np.concatenate(([x[1] - x[0]], (x[2:] - x[:-2]) / 2, [x[-1] - x[-2]])))
            else:
                w_axes.append(np.ones(1))
        return w_axes

    # -- transformations ---------------------------------------------------
    def copy(self):
        return CartesianGrid(self.coords, None if self._weights is None else np.copy(self._weights))

    def scaled(self, scale):
        g = CartesianGrid(self.coords.scaled(scale))
        if self._weights is not None:
            g._weights = self._weights * (abs(scale)**self.ndim if np.isscalar(scale) else np.prod(np.abs(scale)))
        return g

    def shifted(self, shift):
        g = CartesianGrid(self.coords.shifted(shift))
        g._weights = self._weights
        return g

    # -- fields ------------------------------------------------------------
    def zeros(self, tensor_shape=None, dtype=torch.float64, device=None):
        shape = tuple(tensor_shape or ()) + (self.size,)
        return Field(torch.zeros(shape, dtype=_torch_dtype(dtype), device=device or 'cuda'), self)

    def ones(self, tensor_shape=None, dtype=torch.float64, device=None):
        shape = tuple(tensor_shape or ()) + (self.size,)
        return Field(torch.ones(shape, dtype=_torch_dtype(dtype), device=device or 'cuda'), self)

    def empty(self, tensor_shape=None, dtype=torch.float64, device=None):
        shape = tuple(tensor_shape or ()) + (self.size,)
        return Field(torch.empty(shape, dtype=_torch_dtype(dtype), device=device or 'cuda'), self)

    # -- identity ----------------------------------------------------------
    def key(self):
        k = self.coords.key()
        if self._weights is not None:
            k = k + (np.asarray(self._weights).tobytes(),)
        return k

    def __hash__(self):
        return int.from_bytes(hashlib.blake2b(repr(self.key()).encode('latin1'), digest_size=8).digest(), 'little')

    def __eq__(self, other):
        return isinstance(other, CartesianGrid) and self.key() == other.key()

    def __repr__(self):
        return 'CartesianGrid(%s, dims=%s)' % (type(self.coords).__name__, list(self.dims) if self.is_separated else self.size)


def grid_key(grid):
    """Hashable identity of our or the reference's grid (cache key of the propagator instances)."""
    if isinstance(grid, CartesianGrid):
        return grid.key()
    if getattr(grid, 'is_regular', False):
        return ('regular', np.asarray(grid.delta, np.float64).tobytes(), np.asarray(grid.dims, np.int64).tobytes(),
                np.asarray(grid.zero, np.float64).tobytes())
    if getattr(grid, 'is_separated', False):
        return ('separated',) + tuple(np.asarray(c, np.float64).tobytes() for c in grid.separated_coords)
    return ('other', id(grid))


# ---------------------------------------------------------------------------
# Grid factories (hcipy/field/util.py)
# ---------------------------------------------------------------------------


def _tuple(v, n, conv=float):
    if isinstance(v, Iterable) and not isinstance(v, str):
        v = tuple(conv(x) for x in v)
        if len(v) == 1:
            v = v * n
        return v
    return (conv(v),) * n


def _common_size(*args):
    sizes = [len(a) if isinstance(a, Iterable) and not isinstance(a, str) else 1 for a in args]
    return max(sizes)


def make_uniform_grid(dims, extent, center=0, has_center=False):
    """hcipy/field/util.py:68-124."""
    n = _common_size(dims, extent, center)
    dims = np.array(_tuple(dims, n, int), np.int64)
    extent = np.array(_tuple(extent, n), np.float64)
    center = np.array(_tuple(center, n), np.float64)
    delta = extent / dims
    zero = -extent / 2 + center + delta / 2
    if has_center:
        zero = zero - delta / 2 * (1 - dims % 2)
    return CartesianGrid(RegularCoords(delta, dims, zero))


def make_pupil_grid(dims, diameter=1):
    """hcipy/field/util.py:126-163 (always two-dimensional)."""
    return make_uniform_grid(_tuple(dims, 2, int), _tuple(diameter, 2))


def make_focal_grid(q, num_airy, spatial_resolution=None, pupil_diameter=None, focal_length=None, f_number=None,
                    reference_wavelength=None):
    """hcipy/field/util.py:222-318."""
    if isinstance(q, CartesianGrid):
        raise ValueError('The function signature was changed as of HCIPy 0.3.0; use make_focal_grid_from_pupil_grid().')
    if spatial_resolution is None:
        if f_number is None:
            if pupil_diameter is None or focal_length is None:
                if reference_wavelength is None:
                    spatial_resolution = 1.0
                else:
                    raise ValueError('You only supplied a reference wavelength and forgot to supply either an '
                                     'f_number or a (pupil_diameter, focal_length).')
            else:
                f_number = np.asarray(focal_length) / np.asarray(pupil_diameter)
        if spatial_resolution is None:
            if reference_wavelength is None:
                raise ValueError('You supplied an f_number or (pupil_diameter, focal_length), and forgot to supply '
                                 'a reference wavelength.')
            spatial_resolution = np.asarray(f_number) * reference_wavelength
    q = np.broadcast_to(np.asarray(q, np.float64), (2,))
    num_airy = np.broadcast_to(np.asarray(num_airy, np.float64), (2,))
    sr = np.broadcast_to(np.asarray(spatial_resolution, np.float64), (2,))
    delta = sr / q
    dims = np.array([int(2 * n * qq) for n, qq in zip(num_airy, q)], np.int64)
    zero = delta * (-dims / 2 + (dims % 2) * 0.5)
    return CartesianGrid(RegularCoords(delta, dims, zero))


def make_focal_grid_from_pupil_grid(pupil_grid, q=1, num_airy=None, focal_length=1, wavelength=1):
    """hcipy/field/util.py:165-220."""
    from .fourier import make_fft_grid
    if pupil_grid.ndim != 2:
        raise ValueError('The given pupil grid has to be two-dimensional.')
    q = _tuple(q, 2)
    if num_airy is None:
        fov = (1, 1)
    else:
        num_airy = _tuple(num_airy, 2)
        fov = tuple(na / (n / 2) for na, n in zip(num_airy, pupil_grid.dims))
    uv = make_fft_grid(pupil_grid, q, fov)
    return uv.scaled(focal_length * wavelength / (2 * math.pi))


# ---------------------------------------------------------------------------
# Device Field
# ---------------------------------------------------------------------------

_NP_TO_TORCH = {
    np.dtype('float32'): torch.float32, np.dtype('float64'): torch.float64,
    np.dtype('complex64'): torch.complex64, np.dtype('complex128'): torch.complex128,
    np.dtype('bool'): torch.bool, np.dtype('int64'): torch.int64, np.dtype('int32'): torch.int32,
}


def _torch_dtype(dtype):
    if dtype is None or isinstance(dtype, torch.dtype):
        return dtype
    if dtype == 'complex' or dtype is complex:
        return torch.complex128
    if dtype == 'float' or dtype is float:
        return torch.float64
    return _NP_TO_TORCH[np.dtype(dtype)]


def complex_dtype_for(dtype):
    """Complex dtype of the same bit depth (hcipy/fourier/fourier_transform.py:323-346)."""
    if dtype in (torch.float32, torch.complex64, torch.float16, torch.bfloat16):
        return torch.complex64
    return torch.complex128


def as_tensor(x, device='cuda'):
    """A CUDA tensor view/copy of a Field, tensor, numpy array or reference Field."""
    if isinstance(x, Field):
        t = x.data
    elif isinstance(x, torch.Tensor):
        t = x
    else:
        arr = np.asarray(x)
        t = torch.from_numpy(np.ascontiguousarray(arr))
    if t.device.type != 'cuda':
        t = t.to(device, non_blocking=False)
    if t.is_complex() and t.is_conj():  # a lazy conjugate view: the kernels read memory, so materialise it
        t = t.resolve_conj()
    return t


def _unwrap(x):
    return x.data if isinstance(x, Field) else x


class Field(object):
    """Values of a quantity on each point of a grid, stored on the GPU."""
    __slots__ = ('data', 'grid')

    def __init__(self, data, grid=None):
        if isinstance(data, Field):
            if grid is None:
                grid = data.grid
            data = data.data
        self.data = as_tensor(data)
        self.grid = grid

    def __reduce__(self):
        # pickles hold host copies; unpickling uploads them to the device again
        return (Field, (self.data.detach().cpu(), self.grid))

    # -- structure --------------------------------------------------------
    @property
    def tensor_shape(self):
        return tuple(self.data.shape[:-1])

    @property
    def tensor_order(self):
        return self.data.ndim - 1

    @property
    def is_scalar_field(self):
        return self.data.ndim == 1

    @property
    def is_vector_field(self):
        return self.data.ndim == 2

    @property
    def shaped(self):
        """View with the grid axes unflattened: tensor_shape + grid.shape (hcipy/field/field.py:52-65)."""
        if self.grid is None or not self.grid.is_separated:
            return self.data
        return self.data.reshape(self.tensor_shape + tuple(int(d) for d in np.asarray(self.grid.dims)[::-1]))

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def device(self):
        return self.data.device

    @property
    def shape(self):
        return tuple(self.data.shape)

    @property
    def ndim(self):
        return self.data.ndim

    @property
    def size(self):
        return self.data.numel()

    @property
    def real(self):
        return Field(self.data.real, self.grid)

    @property
    def imag(self):
        return Field(self.data.imag, self.grid)

    def conj(self):
        return Field(self.data.conj().resolve_conj(), self.grid)

    def astype(self, dtype, copy=True):
        dt = _torch_dtype(dtype)
        if dt == self.data.dtype and not copy:
            return self
        return Field(self.data.to(dt, copy=copy), self.grid)

    def copy(self):
        return Field(self.data.clone(), self.grid)

    def ravel(self):
        return Field(self.data.reshape(-1), self.grid)

    def reshape(self, *shape):
        return Field(self.data.reshape(*shape), self.grid)

    def numpy(self):
        return self.data.detach().cpu().numpy()

    def cpu(self):
        return self.numpy()

    def __array__(self, dtype=None, copy=None):
        a = self.numpy()
        return a.astype(dtype) if dtype is not None else a

    def __len__(self):
        return self.data.shape[0]

    def __getitem__(self, key):
        key = tuple(_unwrap(k) for k in key) if isinstance(key, tuple) else _unwrap(key)
        return Field(self.data[key], self.grid)

    def __setitem__(self, key, value):
        key = tuple(_unwrap(k) for k in key) if isinstance(key, tuple) else _unwrap(key)
        self.data[key] = _unwrap(value) if not isinstance(value, np.ndarray) else torch.as_tensor(value, device=self.data.device)

    def __repr__(self):
        return 'Field(%r, grid=%r)' % (self.data, self.grid)

    # -- arithmetic (delegates to torch, keeps the grid) -------------------
    def _bin(self, other, op):
        if isinstance(other, np.ndarray) or (hasattr(other, 'grid') and not isinstance(other, Field) and not np.isscalar(other)):
            other = as_tensor(other, self.data.device)
        return Field(op(self.data, _unwrap(other)), self.grid)

    def __add__(self, o): return self._bin(o, torch.add)
    def __radd__(self, o): return self._bin(o, lambda a, b: b + a)
    def __sub__(self, o): return self._bin(o, torch.sub)
    def __rsub__(self, o): return self._bin(o, lambda a, b: b - a)
    def __mul__(self, o): return self._bin(o, torch.mul)
    def __rmul__(self, o): return self._bin(o, lambda a, b: b * a)
    def __truediv__(self, o): return self._bin(o, torch.true_divide)
    def __rtruediv__(self, o): return self._bin(o, lambda a, b: b / a)
    def __pow__(self, o): return self._bin(o, torch.pow)
    def __gt__(self, o): return self._bin(o, lambda a, b: a > b)
    def __ge__(self, o): return self._bin(o, lambda a, b: a >= b)
    def __lt__(self, o): return self._bin(o, lambda a, b: a < b)
    def __le__(self, o): return self._bin(o, lambda a, b: a <= b)
    def __neg__(self): return Field(-self.data, self.grid)
    def __pos__(self): return self
    def __abs__(self): return Field(self.data.abs(), self.grid)

    def _inplace(self, o, op):
        o = _unwrap(o)
        if isinstance(o, np.ndarray):
            o = torch.as_tensor(o, device=self.data.device)
        op(self.data, o)
        return self

    def __iadd__(self, o): return self._inplace(o, torch.Tensor.add_)
    def __isub__(self, o): return self._inplace(o, torch.Tensor.sub_)
    def __imul__(self, o): return self._inplace(o, torch.Tensor.mul_)
    def __itruediv__(self, o): return self._inplace(o, torch.Tensor.div_)


def field_like(data, template):
    return Field(data, template.grid if isinstance(template, Field) else getattr(template, 'grid', None))
