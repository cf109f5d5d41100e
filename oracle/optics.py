"""Propagators and coronagraph chain of the reference, restated in float64 (test infrastructure only)."""
import math

import numpy as np

from . import fourier


def fraunhofer_forward(e, pupil, focal, wavelength=1.0, focal_length=1.0):
    """hcipy/propagation/fraunhofer.py:32-71: MFT onto output_grid scaled by 2 pi/(f lambda), times 1/(i f lambda)."""
    uv = focal.scaled(2 * np.pi / (focal_length * wavelength))
    x, y = pupil.separated_coords
    u, v = uv.separated_coords
    norm = 1 / (1j * focal_length * wavelength)
    return fourier.mft_forward(e, x, y, u, v, pupil.weights) * norm


def fraunhofer_backward(f, pupil, focal, wavelength=1.0, focal_length=1.0):
    """hcipy/propagation/fraunhofer.py:73-88: inverse MFT divided by the norm factor."""
    uv = focal.scaled(2 * np.pi / (focal_length * wavelength))
    x, y = pupil.separated_coords
    u, v = uv.separated_coords
    norm = 1 / (1j * focal_length * wavelength)
    w_out = uv.weights
    return fourier.mft_backward(f, x, y, u, v, w_out) / norm


def lyot_forward(e, pupil, fpm_grid, fpm, stop=None, wavelength=1.0, focal_length=1.0):
    """hcipy/coronagraphy/lyot.py:66-92 (Babinet form)."""
    ef = fraunhofer_forward(e, pupil, fpm_grid, wavelength, focal_length)
    ef = ef - np.asarray(fpm) * ef
    lyot = fraunhofer_backward(ef, pupil, fpm_grid, wavelength, focal_length)
    lyot = np.asarray(e) - lyot
    if stop is not None:
        lyot = lyot * np.asarray(stop)
    return lyot


def apodize(e, a, adjoint=False):
    """hcipy/optics/apodization.py:25-35."""
    return np.asarray(e) * (np.conj(a) if adjoint else a)


def dm_surface(influence, actuators):
    """ModeBasis.linear_combination (hcipy/mode_basis/mode_basis.py:239-258): influence^T . a."""
    return np.asarray(influence).T @ np.asarray(actuators) if np.asarray(influence).shape[0] == len(actuators) \
        else np.asarray(influence) @ np.asarray(actuators)


def dm_forward(e, surface, wavelength):
    """hcipy/optics/deformable_mirror.py:200-217: E * exp(2 i k S)."""
    k = 2 * np.pi / wavelength
    return np.asarray(e) * np.exp(2j * k * np.asarray(surface))


def circular_aperture(grid, diameter):
    """hcipy/aperture/generic.py:31-44: 1 where x^2 + y^2 <= (diameter / 2)^2."""
    x, y = grid.coords()
    return ((x**2 + y**2) <= (diameter / 2)**2).astype(np.float64)


def surface_apodize(e, sag, n, wavelength):
    """hcipy/optics/apodization.py:88-93: E * exp(i (n - 1) sag k)."""
    return np.asarray(e) * np.exp(1j * (n - 1) * np.asarray(sag) * (2 * np.pi / wavelength))


class PyramidOptics(object):
    """hcipy/wavefront_sensing/pyramid.py:94-181: lens, circular field stop, glass pyramid (SurfaceApodizer), lens."""

    def __init__(self, pupil, out_grid, separation, pupil_diameter, wavelength_0, refractive_index):
        from .grids import make_pupil_grid
        d_in = pupil.delta * pupil.dims
        d_out = out_grid.delta * out_grid.dims
        q = np.ceil(max(np.max(d_out / d_in), 2))  # pyramid.py:129-135
        self.num_airy = np.max(pupil.shape) / 2
        num_pixels = 2 * int(self.num_airy * q)
        self.focal = make_pupil_grid(num_pixels, 2 * (wavelength_0 / pupil_diameter) * self.num_airy)
        self.pupil, self.out_grid = pupil, out_grid
        self.separation, self.wavelength_0, self.refractive_index = separation, wavelength_0, refractive_index
        self.stop = circular_aperture(self.focal, 2 * self.num_airy * wavelength_0 / pupil_diameter)
        self.sag = self.sag_function(*self.focal.coords())

    def sag_function(self, x, y):
        """pyramid.py:148 (and :54-55): -separation / (2 (n(lambda_0) - 1)) (|x| + |y|)."""
        return -self.separation / (2 * (self.refractive_index(self.wavelength_0) - 1)) * (np.abs(x) + np.abs(y))

    def to_focal(self, e, wavelength):
        """pyramid.py:176: the first lens and the field stop."""
        return fraunhofer_forward(e, self.pupil, self.focal, wavelength) * self.stop

    def forward(self, e, wavelength, sag=None):
        """pyramid.py:175-181, with another pyramid sag when given."""
        f = surface_apodize(self.to_focal(e, wavelength), self.sag if sag is None else sag,
                            self.refractive_index(wavelength), wavelength)
        return fraunhofer_forward(f, self.focal, self.out_grid, wavelength)


def tip_tilt_forward(e, pupil, command, wavelength):
    """hcipy/optics/tip_tilt_mirror.py with deformable_mirror.py:200-217: the surface x a_0 + y a_1 reflected,
    E exp(2 i k S)."""
    x, y = pupil.coords()
    return dm_forward(e, x * command[0] + y * command[1], wavelength)


def modulation_positions(modulation, num_steps):
    """hcipy/wavefront_sensing/pyramid.py:39-44."""
    theta = np.linspace(0, 2 * np.pi, num_steps, endpoint=False)
    return np.stack((modulation / 2 * np.cos(theta), modulation / 2 * np.sin(theta)), axis=1)


def modulated_pyramid_forward(optics, e, wavelength, modulation, num_steps, fast=False):
    """hcipy/wavefront_sensing/pyramid.py:65-88, both methods: (num_steps, npix_out).

    Tip-tilt method: the pyramid optics applied to the input tilted to each modulation position.  Fast method:
    one focal-plane field through the stop, then per step the pyramid sag on the focal grid shifted by twice the
    position, sampled 4x per axis and averaged (pyramid.py:50-63), and the second lens."""
    pos = modulation_positions(modulation, num_steps)
    if not fast:
        return np.stack([optics.forward(tip_tilt_forward(e, optics.pupil, p, wavelength), wavelength) for p in pos])
    focal = optics.to_focal(e, wavelength)
    n = optics.refractive_index(wavelength)
    out = []
    for p in pos:
        sag = fourier.supersampled_mean(optics.sag_function, optics.focal.shifted(2 * p), 4)
        out.append(fraunhofer_forward(surface_apodize(focal, sag, n, wavelength), optics.focal, optics.out_grid,
                                      wavelength))
    return np.stack(out)


def vortex_mask(charge):
    """hcipy/coronagraphy/vortex.py:13-14: exp(i charge theta), zero inside make_circular_aperture(1e-9)."""
    def mask(grid):
        x, y = grid.coords()
        return np.exp(1j * charge * np.arctan2(y, x)) * (1 - (x**2 + y**2 <= (1e-9 / 2)**2))
    return mask


def retarder_jones(retardance, fast_axis):
    """hcipy/optics/polarization.py:141-160 for a linear retarder (circularity 0): the (2, 2, n) Jones matrix."""
    plus, minus = np.exp(1j * retardance / 2), np.exp(-1j * retardance / 2)
    c, s = np.cos(fast_axis), np.sin(fast_axis)
    j11 = plus * c**2 + minus * s**2
    j12 = (plus - minus) * np.exp(-1j * 0) * c * s
    j21 = (plus - minus) * np.exp(1j * 0) * c * s
    j22 = plus * s**2 + minus * c**2
    return np.array([[j11, j12], [j21, j22]])


def vector_vortex_mask(charge, retardance):
    """hcipy/coronagraphy/vortex.py:94-100: the retarder with fast axis charge / 2 * theta, zero at the centre."""
    def mask(grid):
        x, y = grid.coords()
        j = retarder_jones(retardance, charge / 2 * np.arctan2(y, x))
        return j * (1 - (x**2 + y**2 <= (1e-9 / 2)**2))
    return mask


def _field_dot(a, b):
    """hcipy/field/field.py field_dot for a (2, 2, n) matrix field and a (2, n) or (2, 2, n) field."""
    return np.einsum('ij...n,j...n->i...n', a, b)


class MultiScaleOptics(object):
    """hcipy/coronagraphy/multi_scale.py:62-161 (and, for a (2, 2, n) Jones-matrix mask, the vector vortex's
    vortex.py:79-246): level 0 a Fourier filter at q = 2, level i > 0 a window scaling_factor times finer with the
    coarser levels' contribution subtracted, propagated at unit wavelength and focal length."""

    def __init__(self, pupil, complex_mask, q=1024, scaling_factor=4, window_size=32):
        from scipy.signal import windows
        from .grids import make_focal_grid
        self.pupil = pupil
        diameter = pupil.dims * pupil.delta
        levels = int(math.ceil(math.log(q / 2) / math.log(scaling_factor))) + 1
        qs = [2 * scaling_factor**i for i in range(levels)]
        num_airys = [tuple(n / 2 for n in pupil.dims)]
        for i in range(1, levels):
            num_airys.append(tuple(n * window_size / (2 * qs[i - 1] * n) for n in num_airys[i - 1]))
        self.focal_grids, self.masks = [], []
        for i in range(levels):
            focal = make_focal_grid(qs[i], num_airys[i], spatial_resolution=1 / diameter)
            m = np.asarray(complex_mask(focal), np.complex128)
            if i != levels - 1:
                w = np.outer(windows.tukey(window_size, 1, False), windows.tukey(window_size, 1, False))
                w = np.pad(w, tuple((n_foc - n_w) // 2 for n_foc, n_w in zip(focal.shape, w.shape)), 'constant')
                m = m * (1 - w.ravel())
            for j in range(i):
                fft = fourier.FFTPlan(self.focal_grids[j])
                x, y = focal.separated_coords
                u, v = fft.output_grid.separated_coords
                back = np.array([fourier.mft_backward(fft.forward(mj), x, y, u, v, fft.output_grid.weights)
                                 for mj in self.masks[j].reshape(-1, self.focal_grids[j].size)])
                m = m - back.reshape(m.shape)
            self.focal_grids.append(focal)
            self.masks.append(m)
        self.jones = self.masks[0].ndim == 3
        tf = self.masks[0].reshape(-1, self.focal_grids[0].size)
        self.filters = [fourier.FourierFilterPlan(pupil, t, qs[0]) for t in tf]

    def _filter(self, e, adjoint):
        if not self.jones:
            return self.filters[0].apply(e, adjoint)
        # fourier_operations.py:112-121: FFT of every entry, the matrix product with the transfer function (its
        # conjugate transpose for the adjoint), inverse FFT
        plan = self.filters[0]
        tfs = np.array([f.tf for f in self.filters]).reshape((2, 2) + plan.internal_grid.shape)
        if adjoint:
            tfs = np.conj(np.swapaxes(tfs, 0, 1))
        lead = e.shape[:-1]
        spec = []
        for ej in e.reshape((-1, e.shape[-1])):
            f = np.zeros(plan.internal_grid.shape, dtype=np.complex128)
            f[plan.cutout] = ej.reshape(plan.shape_in)
            spec.append(np.fft.fftn(f))
        spec = np.array(spec).reshape(lead + plan.internal_grid.shape)
        prod = np.einsum('ij...,j...->i...', tfs, spec)
        out = [np.fft.ifftn(p)[plan.cutout].ravel() for p in prod.reshape((-1,) + plan.internal_grid.shape)]
        return np.array(out).reshape(lead + (plan.shape_in[0] * plan.shape_in[1],))

    def propagate(self, e, adjoint=False):
        """Lyot plane of e (multi_scale.py:95-128, vortex.py:160-202), or with ``adjoint`` the backward
        propagation (multi_scale.py:130-161, vortex.py:204-246).  For a Jones-matrix mask a scalar e is taken as
        e times the identity."""
        e = np.asarray(e, np.complex128)
        if self.jones and e.ndim == 1:
            e = np.array([[e, np.zeros_like(e)], [np.zeros_like(e), e]])
        lyot = self._filter(e, adjoint)
        for focal, m in zip(self.focal_grids[1:], self.masks[1:]):
            f = np.array([fraunhofer_forward(ek, self.pupil, focal) for ek in e.reshape((-1, e.shape[-1]))])
            f = f.reshape(e.shape[:-1] + (focal.size,))
            m = np.conj(m) if adjoint else m  # vortex.py:240: the conjugate, not the conjugate transpose
            f = _field_dot(m, f) if self.jones else m * f
            back = np.array([fraunhofer_backward(fk, self.pupil, focal) for fk in f.reshape((-1, focal.size))])
            lyot = lyot + back.reshape(lyot.shape)
        return lyot


def stokes_parameters(jones, stokes):
    """hcipy/optics/wavefront.py:103-235 for a partially polarised wavefront: (I, Q, U, V) of the (2, 2, n)
    Jones-matrix field acting on the input Stokes vector, through the Mueller matrix A (J kron J*) A^-1."""
    a = np.array([[1, 0, 0, 1], [1, 0, 0, -1], [0, 1, 1, 0], [0, 1j, -1j, 0]])
    ainv = np.linalg.inv(a)
    j = np.moveaxis(np.asarray(jones), -1, 0)
    kron = np.einsum('nij,nkl->nikjl', j, np.conj(j)).reshape(-1, 4, 4)
    mueller = np.einsum('ab,nbc,cd->nad', a, kron, ainv)
    return np.einsum('nab,b->an', mueller, np.asarray(stokes, np.float64)).real


def intensity(e):
    """hcipy/optics/wavefront.py:113-143 scalar branch."""
    return np.abs(e)**2


class LyotChain(object):
    """Lyot coronagraph plus final imaging with the MFT matrices computed once, as the reference does by
    default (``precompute_matrices=True``, hcipy/config/default_config.yaml:18-20; matrix_fourier_transform.py:67-111).

    This is the CPU port timed as the baseline: the same GEMM order as the
    reference (matrix_fourier_transform.py:165-172 and :219-220), element-wise
    steps of lyot.py:79-90, in the requested complex dtype.
    """

    def __init__(self, pupil, fpm_grid, focal, fpm, stop, wavelength=1.0, dtype=np.complex128):
        self.dtype = np.dtype(dtype)
        rdt = np.float32 if self.dtype == np.complex64 else np.float64
        x, y = pupil.separated_coords
        self.shape_in = pupil.shape
        self.fpm_shape = fpm_grid.shape
        self.focal_shape = focal.shape
        uv = fpm_grid.scaled(2 * np.pi / wavelength)
        u, v = uv.separated_coords
        m1, m2 = fourier.mft_matrices(x, y, u, v)
        self.m1 = m1.astype(self.dtype)
        self.m2 = m2.astype(self.dtype)
        self.m1h = np.ascontiguousarray(m1.conj().T).astype(self.dtype)
        self.m2h = np.ascontiguousarray(m2.conj().T).astype(self.dtype)
        uf, vf = focal.scaled(2 * np.pi / wavelength).separated_coords
        f1, f2 = fourier.mft_matrices(x, y, uf, vf)
        self.f1 = f1.astype(self.dtype)
        self.f2 = f2.astype(self.dtype)
        norm = 1 / (1j * wavelength)
        self.a_fwd = self.dtype.type(pupil.weights * norm)
        self.a_bwd = self.dtype.type(uv.weights / (2 * np.pi)**2 / norm)
        self.a_img = self.dtype.type(pupil.weights * norm)
        self.one_minus_fpm = (1 - np.asarray(fpm)).reshape(self.fpm_shape).astype(rdt)
        self.stop = np.asarray(stop).reshape(self.shape_in).astype(rdt)

    def lyot(self, e):
        e = np.asarray(e, self.dtype).reshape(self.shape_in)
        ef = (self.m1 @ (e @ self.m2)) * self.a_fwd
        ef *= self.one_minus_fpm
        lp = ((self.m1h @ ef) @ self.m2h) * self.a_bwd
        return ((e - lp) * self.stop).ravel()

    def image(self, lyot_field):
        lp = np.asarray(lyot_field, self.dtype).reshape(self.shape_in)
        return ((self.f1 @ (lp @ self.f2)) * self.a_img).ravel()

    def __call__(self, e):
        return self.image(self.lyot(e))

    def image_adjoint(self, g):
        """Conjugate transpose of ``image``: conj(a_img) F1^H g F2^H."""
        g = np.asarray(g, self.dtype).reshape(self.focal_shape)
        return (np.conj(self.a_img) * (self.f1.conj().T @ (g @ self.f2.conj().T))).ravel()

    def lyot_adjoint(self, g):
        """Conjugate transpose of ``lyot``: u - conj(a_fwd) M1^H [(1 - M) conj(a_bwd) M1 u M2] M2^H, u = S g."""
        u = np.asarray(g, self.dtype).reshape(self.shape_in) * self.stop
        v = (self.m1 @ (u @ self.m2)) * np.conj(self.a_bwd)
        v *= self.one_minus_fpm
        w = ((self.m1h @ v) @ self.m2h) * np.conj(self.a_fwd)
        return (u - w).ravel()


def dm_lyot_loss_grad(chain, influence, aperture, actuators, roi, wavelength=1.0):
    """Loss sum_roi |image|^2 of one command vector through DM -> Lyot -> image, and its gradient in the
    actuators by the adjoint chain (torch's convention: dL/d(conj z) times 2 for complex intermediates).

    influence: (npix x nact) scipy sparse or dense matrix; the DM reflects E exp(2ik S)
    (hcipy/optics/deformable_mirror.py:200-217).
    """
    k = 2 * np.pi / wavelength
    s = influence @ np.asarray(actuators, np.float64)
    e = np.asarray(aperture) * np.exp(2j * k * s)
    img = chain(e)
    roi = np.asarray(roi, np.float64)
    loss = float(np.sum(roi * np.abs(img)**2))
    g_e = chain.lyot_adjoint(chain.image_adjoint(2 * roi * img))
    g_s = 2 * k * np.imag(np.conj(e) * g_e)
    return loss, influence.T @ g_s
