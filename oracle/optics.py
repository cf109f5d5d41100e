"""Propagators and coronagraph chain of the reference, restated in float64 (test infrastructure only)."""
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
