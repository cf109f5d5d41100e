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
