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
