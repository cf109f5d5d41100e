"""Regular-grid algebra of the reference, restated (test infrastructure only).

A regular grid is described by ``(delta, dims, zero)`` per axis, axis 0 = x.
Coordinates along axis i are ``zero[i] + delta[i] * arange(dims[i])``; a flat
field is stored y-major (C order of shape ``(dims[1], dims[0])``).
"""
import math

import numpy as np


class RegularGrid(object):
    def __init__(self, delta, dims, zero):
        self.delta = np.asarray(delta, dtype=np.float64)
        self.dims = np.asarray(dims, dtype=np.int64)
        self.zero = np.asarray(zero, dtype=np.float64)

    @property
    def ndim(self):
        return len(self.dims)

    @property
    def shape(self):
        return tuple(int(d) for d in self.dims[::-1])

    @property
    def size(self):
        return int(np.prod(self.dims))

    @property
    def weights(self):
        # hcipy/field/cartesian_grid.py:168-170: regular grids weigh prod(delta).
        return float(np.prod(self.delta))

    def axis(self, i):
        return self.zero[i] + self.delta[i] * np.arange(self.dims[i])

    @property
    def separated_coords(self):
        return [self.axis(i) for i in range(self.ndim)]

    def coords(self):
        """Flat coordinate arrays in field order (x varies fastest)."""
        axes = self.separated_coords
        mesh = np.meshgrid(*axes, indexing='xy') if self.ndim == 2 else axes
        return [m.ravel() for m in mesh]

    def scaled(self, s):
        # hcipy/field/cartesian_grid.py:83-104 (coords *= scale).
        return RegularGrid(self.delta * s, self.dims, self.zero * s)

    def shifted(self, s):
        return RegularGrid(self.delta, self.dims, self.zero + np.asarray(s, np.float64))


def make_uniform_grid(dims, extent, center=0, has_center=False):
    # hcipy/field/util.py:68-124.
    dims = np.broadcast_to(np.asarray(dims, np.int64), (2,)) if np.ndim(dims) == 0 else np.asarray(dims, np.int64)
    n = len(dims)
    extent = np.broadcast_to(np.asarray(extent, np.float64), (n,))
    center = np.broadcast_to(np.asarray(center, np.float64), (n,))
    delta = extent / dims
    zero = -extent / 2 + center + delta / 2
    if has_center:
        zero = zero - delta / 2 * (1 - dims % 2)
    return RegularGrid(delta, dims, zero)


def make_pupil_grid(dims, diameter=1):
    # hcipy/field/util.py:126-163.
    return make_uniform_grid(np.broadcast_to(np.asarray(dims), (2,)), np.broadcast_to(np.asarray(diameter, np.float64), (2,)))


def make_focal_grid(q, num_airy, spatial_resolution=1.0):
    # hcipy/field/util.py:222-318 (normalised units when spatial_resolution is 1).
    q = np.broadcast_to(np.asarray(q, np.float64), (2,))
    num_airy = np.broadcast_to(np.asarray(num_airy, np.float64), (2,))
    sr = np.broadcast_to(np.asarray(spatial_resolution, np.float64), (2,))
    delta = sr / q
    dims = np.array([int(2 * n * qq) for n, qq in zip(num_airy, q)], np.int64)
    zero = delta * (-dims / 2 + (dims % 2) * 0.5)
    return RegularGrid(delta, dims, zero)


def make_fft_grid(input_grid, q=1, fov=1, shift=0):
    # hcipy/fourier/fast_fourier_transform.py:23-62.
    n = input_grid.ndim
    q = np.broadcast_to(np.asarray(q, np.float64), (n,))
    fov = np.broadcast_to(np.asarray(fov, np.float64), (n,))
    shift = np.broadcast_to(np.asarray(shift, np.float64), (n,))
    q = np.array([round(qi * d) / d for qi, d in zip(q, input_grid.dims)])
    delta = np.array([float((2 * math.pi / (d * s)) / qi) for d, s, qi in zip(input_grid.delta, input_grid.dims, q)])
    dims = np.array([int(d * f * qi) for d, f, qi in zip(input_grid.dims, fov, q)], np.int64)
    zero = np.array([float(di * (-dim / 2 + (dim % 2) * 0.5) + si) for di, dim, si in zip(delta, dims, shift)])
    return RegularGrid(delta, dims, zero)
