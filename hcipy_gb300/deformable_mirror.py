"""Deformable mirror (hcipy/optics/deformable_mirror.py) with its surface and phase on the device.

Influence functions are built on the host once, as in the reference (they are plan-time data): Gaussian pokes
(hcipy/mode_basis/gaussian_pokes.py:5-54) on the BMC actuator grid (deformable_mirror.py:13-38), cut off at
``cutoff`` actuator pitches, with the cut-off value subtracted, stored sparse.  On the device the basis is a
CSR/CSC pair (``kernels.SparseBasis``): the surface of a batch of command vectors is one sparse product, the
reflection E exp(+-2ik S) one phase kernel, and both have adjoints, so ``DeformableMirror.forward`` is
differentiable in the actuators when they are a tensor with ``requires_grad``.
"""
import numpy as np
import scipy.sparse
import torch

from .field import CartesianGrid, RegularCoords, Field, as_tensor, make_uniform_grid
from .kernels import SparseBasis
from .optics import OpticalElement


class ModeBasis(object):
    """A set of modes on a grid as a (npix x nmodes) matrix, dense or scipy-sparse (hcipy/mode_basis/mode_basis.py).

    Only what the deformable mirror needs: the matrix, the grid, the number of modes, ``linear_combination``.
    """

    def __init__(self, transformation_matrix, grid=None):
        if isinstance(transformation_matrix, (list, tuple)):
            cols = [scipy.sparse.csr_matrix(np.asarray(m).reshape(1, -1)) if not scipy.sparse.issparse(m)
                    else scipy.sparse.csr_matrix(m).reshape(1, -1) for m in transformation_matrix]
            transformation_matrix = scipy.sparse.vstack(cols).T.tocsr()
        self._transformation_matrix = transformation_matrix
        self.grid = grid
        self._device = {}

    def __getstate__(self):
        state = dict(self.__dict__)
        state['_device'] = {}  # device copies are rebuilt on first use
        return state

    @property
    def transformation_matrix(self):
        return self._transformation_matrix

    @property
    def is_sparse(self):
        return scipy.sparse.issparse(self._transformation_matrix)

    @property
    def num_modes(self):
        return self._transformation_matrix.shape[1]

    def __len__(self):
        return self.num_modes

    def device_basis(self, device, dtype):
        key = (str(device), dtype)
        b = self._device.get(key)
        if b is None:
            m = self._transformation_matrix
            b = SparseBasis(m if self.is_sparse else scipy.sparse.csr_matrix(np.asarray(m)), device, dtype)
            self._device[key] = b
        return b

    def linear_combination(self, coefficients):
        """sum_i c_i mode_i on the device (mode_basis.py:239-258); coefficients may carry a leading batch."""
        c = torch.as_tensor(np.asarray(coefficients, np.float64)) if not isinstance(coefficients, torch.Tensor) \
            else coefficients
        dev = torch.device('cuda')
        b = self.device_basis(dev, torch.float64 if c.dtype == torch.float64 else torch.float32)
        return Field(b.apply(c.to(dev)), self.grid)


def make_actuator_positions(num_actuators_across_pupil, actuator_spacing, x_tilt=0, y_tilt=0, z_tilt=0):
    """Actuator positions in the BMC convention (deformable_mirror.py:13-38); returns (x, y) float64 arrays."""
    extent = actuator_spacing * num_actuators_across_pupil
    g = make_uniform_grid(num_actuators_across_pupil, [extent, extent])
    x, y = g.points[:, 0] * np.cos(y_tilt), g.points[:, 1] * np.cos(x_tilt)
    if z_tilt != 0:
        c, s = np.cos(z_tilt), np.sin(z_tilt)
        x, y = c * x - s * y, s * x + c * y
    return x, y


def _grid_xy(grid):
    if hasattr(grid, 'points'):
        p = np.asarray(grid.points)
        return p[:, 0], p[:, 1]
    xs, ys = grid.separated_coords
    xx, yy = np.meshgrid(xs, ys)
    return xx.ravel(), yy.ravel()


def make_gaussian_influence_functions(pupil_grid, num_actuators_across_pupil, actuator_spacing, crosstalk=0.15,
                                      cutoff=3, x_tilt=0, y_tilt=0, z_tilt=0, oversampling=1):
    """Gaussian influence functions (deformable_mirror.py:40-93 with gaussian_pokes.py:5-54).

    sigma = spacing / sqrt(-2 ln crosstalk); each poke is exp(-r^2 / 2 sigma^2) - exp(-cutoff'^2 / 2), zero
    beyond cutoff' sigma = cutoff * spacing, evaluated on the (tilt-transformed) pupil grid and averaged over
    oversampling^2 sub-pixel samples.  Returns a sparse ``ModeBasis``.
    """
    ax, ay = make_actuator_positions(num_actuators_across_pupil, actuator_spacing)
    sigma = actuator_spacing / np.sqrt(-2 * np.log(crosstalk))
    cut = actuator_spacing / sigma * cutoff
    offset = np.exp(-0.5 * cut**2)
    os_ = int(round(oversampling))
    delta = np.asarray(getattr(pupil_grid, 'delta', [0.0, 0.0]), np.float64)
    if os_ > 1:
        offs = (np.arange(os_) - (os_ - 1) / 2) / os_
        dithers = [(dx * delta[0], dy * delta[1]) for dy in offs for dx in offs]
    else:
        dithers = [(0.0, 0.0)]
    c, s = np.cos(-z_tilt), np.sin(-z_tilt)
    norm = 1.0 / (np.cos(x_tilt) * np.cos(y_tilt))
    untilted = x_tilt == 0 and y_tilt == 0 and z_tilt == 0
    if untilted and getattr(pupil_grid, 'is_separated', False):
        xs, ys = (np.asarray(v, np.float64) for v in pupil_grid.separated_coords)
        nx = xs.size
    else:
        px, py = _grid_xy(pupil_grid)
    npix = pupil_grid.size
    reach = cut * sigma + np.max(np.abs(delta))
    rows, cols, vals = [], [], []
    for a in range(ax.size):
        if untilted and getattr(pupil_grid, 'is_separated', False):
            # only the pixels in the poke's bounding box can be nonzero
            i0, i1 = np.searchsorted(xs, [ax[a] - reach, ax[a] + reach])
            j0, j1 = np.searchsorted(ys, [ay[a] - reach, ay[a] + reach])
            bx, by = np.meshgrid(xs[i0:i1], ys[j0:j1])
            bx, by = bx.ravel(), by.ravel()
            idx = (np.arange(j0, j1)[:, None] * nx + np.arange(i0, i1)[None, :]).ravel()
        else:
            bx, by, idx = px, py, np.arange(npix)
        acc = np.zeros(idx.size)
        for dx, dy in dithers:
            # evaluated grid: pupil grid scaled by 1/cos(tilt), rotated by -z_tilt (deformable_mirror.py:78-84)
            gx = (bx + dx) / np.cos(y_tilt)
            gy = (by + dy) / np.cos(x_tilt)
            rx, ry = c * gx - s * gy, s * gx + c * gy
            r2 = (rx - ax[a])**2 + (ry - ay[a])**2
            p = np.exp(-0.5 * r2 / sigma**2) - offset
            p[r2 > (cut * sigma)**2] = 0
            acc += p
        acc *= norm / len(dithers)
        nz = np.nonzero(acc)[0]
        rows.append(idx[nz])
        cols.append(np.full(nz.size, a))
        vals.append(acc[nz])
    m = scipy.sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                shape=(npix, ax.size))
    m.sort_indices()
    return ModeBasis(m, pupil_grid)


def find_illuminated_actuators(basis, aperture, power_cutoff=0.1):
    """Modes with at least ``power_cutoff`` of their power inside the aperture (deformable_mirror.py:135-157)."""
    m = basis.transformation_matrix
    m = scipy.sparse.csc_matrix(m) if scipy.sparse.issparse(m) else np.asarray(m)
    a = np.asarray(aperture.data.cpu() if isinstance(aperture, Field) else aperture).ravel() > 0
    sq = m.multiply(m) if scipy.sparse.issparse(m) else np.abs(m)**2
    total = np.asarray(sq.sum(axis=0)).ravel()
    masked = np.asarray(sq[a].sum(axis=0)).ravel()
    keep = masked >= power_cutoff * total
    return ModeBasis(m[:, keep].tocsr() if scipy.sparse.issparse(m) else m[:, keep], basis.grid)


class DeformableMirror(OpticalElement):
    """A deformable mirror from influence functions (deformable_mirror.py:159-300).

    ``actuators`` may be a numpy array (nact,), or a tensor (..., nact) holding a batch of command vectors;
    the surface and the reflected wavefronts then carry the same leading batch.  A tensor with
    ``requires_grad`` makes ``forward``/``backward`` differentiable in the actuators.
    """

    def __init__(self, influence_functions, dtype=torch.float32):
        if not isinstance(influence_functions, ModeBasis):
            grid = getattr(influence_functions, 'grid', None)
            mat = getattr(influence_functions, 'transformation_matrix', influence_functions)
            influence_functions = ModeBasis(mat, grid)
        self._influence_functions = influence_functions
        self.dtype = dtype
        self.input_grid = influence_functions.grid
        self._actuators = np.zeros(len(influence_functions))
        self._cache_key = None
        self._surface = None

    @property
    def influence_functions(self):
        return self._influence_functions

    @influence_functions.setter
    def influence_functions(self, influence_functions):
        self._influence_functions = influence_functions
        self._cache_key = None

    @property
    def num_actuators(self):
        return len(self._influence_functions)

    @property
    def actuators(self):
        return self._actuators

    @actuators.setter
    def actuators(self, actuators):
        self._actuators = actuators

    def flatten(self):
        self._actuators = np.zeros(len(self._influence_functions))

    def random(self, rms):
        self._actuators = np.random.randn(len(self._influence_functions)) * rms

    def _basis(self, dtype):
        return self._influence_functions.device_basis(torch.device('cuda'), dtype)

    def _surface_tensor(self, dtype=None):
        dtype = dtype or self.dtype
        a = self._actuators
        if isinstance(a, torch.Tensor):
            if torch.is_grad_enabled() and a.requires_grad:
                from .autograd import influence_apply
                return influence_apply(self._basis(dtype), a.to('cuda'))
            return self._basis(dtype).apply(a.detach().to('cuda'))
        a = np.asarray(a, np.float64)
        # deformable_mirror.py:251-262: the surface is cached until the actuators change.
        key = (a.tobytes(), dtype)
        if self._cache_key != key:
            self._surface = self._basis(dtype).apply(torch.from_numpy(a))
            self._cache_key = key
        return self._surface

    @property
    def surface(self):
        """The surface in meters (a device Field)."""
        return Field(self._surface_tensor(), self.input_grid)

    @property
    def opd(self):
        return Field(2 * self._surface_tensor(), self.input_grid)

    def phase_for(self, wavelength):
        return Field(self._surface_tensor() * (4 * np.pi / wavelength), self.input_grid)

    def _reflect(self, wavefront, sign):
        e = as_tensor(wavefront.electric_field)
        rdt = torch.float64 if e.dtype == torch.complex128 else torch.float32
        s = self._surface_tensor(rdt)
        scale = sign * 2 * (2 * np.pi / wavefront.wavelength)
        if torch.is_grad_enabled() and (s.requires_grad or e.requires_grad):
            from .autograd import phase_apply
            out = phase_apply(e, s, scale)
        else:
            from .kernels import apply_phase
            out = apply_phase(e, s, scale)
        return wavefront._carry(Field(out, wavefront.electric_field.grid))

    def forward(self, wavefront):
        """E exp(2ik S) (deformable_mirror.py:200-217)."""
        return self._reflect(wavefront, +1.0)

    def backward(self, wavefront):
        """E exp(-2ik S) (deformable_mirror.py:219-238)."""
        return self._reflect(wavefront, -1.0)


class TipTiltMirror(DeformableMirror):
    """A tip-tilt mirror (hcipy/optics/tip_tilt_mirror.py): a deformable mirror whose two modes are the input grid's
    x and y coordinates, so its two actuators are the surface's slopes along x and y (OPD-controlled, as in the
    reference).  A tensor of commands of shape (..., 2) reflects the wavefront at every command in one launch."""

    def __init__(self, input_grid, dtype=torch.float32):
        x, y = _grid_xy(input_grid)
        super(TipTiltMirror, self).__init__(ModeBasis(np.stack([x, y], axis=1), input_grid), dtype)
        self.input_grid = input_grid
        self._actuators = np.zeros((2,))
