"""Infinite-phase-screen extrusion and quintic sub-pixel shift, restated (test infrastructure only)."""
import math

import numpy as np


def quintic_weights(shift):
    """7-tap quintic B-spline kernel, hcipy/_math/subpixel_shift.py:7-35."""
    f = abs(shift)
    b = np.empty(6)
    for i, offset in enumerate([2.0 + f, 1.0 + f, f, 1.0 - f, 2.0 - f, 3.0 - f]):
        s = 0.0
        x = offset + 3.0
        for c in (1.0, -6.0, 15.0, -20.0, 15.0, -6.0, 1.0):
            if x > 0.0:
                s += c * x**5
            x -= 1.0
        b[i] = s / 120.0
    if shift >= 0:
        return np.array([0.0, b[0], b[1], b[2], b[3], b[4], b[5]])
    return np.array([b[5], b[4], b[3], b[2], b[1], b[0], 0.0])


def separable_convolve(img, kernel_row, kernel_col):
    """Clamp-to-edge separable convolution, rows then columns (subpixel_shift.py:38-116)."""
    img = np.asarray(img, dtype=np.float64)
    h, w = img.shape
    r = len(kernel_row) // 2
    cols = np.clip(np.arange(w)[:, None] + np.arange(-r, r + 1)[None, :], 0, w - 1)
    tmp = (img[:, cols] * kernel_row[None, None, :]).sum(-1)
    r = len(kernel_col) // 2
    rows = np.clip(np.arange(h)[:, None] + np.arange(-r, r + 1)[None, :], 0, h - 1)
    return (tmp[rows, :] * kernel_col[None, :, None]).sum(1)


def subpixel_shift(img, row_shift, col_shift):
    """subpixel_shift.py:306-343."""
    if not (-0.5 <= row_shift <= 0.5) or not (-0.5 <= col_shift <= 0.5):
        raise ValueError('row_shift and col_shift must be in [-0.5, 0.5]')
    return separable_convolve(img, quintic_weights(col_shift), quintic_weights(row_shift))


def extrude(screen, shape, where, a_mat, b_mat, stencil_idx, noise):
    """One autoregressive row/column, hcipy/atmosphere/infinite_atmospheric_layer.py:216-259.

    ``screen`` is the flat achromatic screen (y-major), ``noise`` the normal
    draws of this step (length ``b_mat.shape[1]``).  Returns the new flat screen.
    """
    screen = np.asarray(screen, np.float64)
    flip = where in ('top', 'right')
    s1 = screen[::-1] if flip else screen
    new_slice = a_mat.dot(s1[stencil_idx]) + b_mat.dot(noise)
    s2 = screen.reshape(shape)
    out = np.empty_like(s2)
    if where == 'top':
        out[:-1, :] = s2[1:, :]
        out[-1, :] = new_slice[::-1]
    elif where == 'bottom':
        out[0, :] = new_slice
        out[1:, :] = s2[:-1, :]
    elif where == 'left':
        out[:, 0] = new_slice
        out[:, 1:] = s2[:, :-1]
    elif where == 'right':
        out[:, :-1] = s2[:, 1:]
        out[:, -1] = new_slice[::-1]
    else:
        raise ValueError('Invalid value for `where`')
    return out.ravel()


def evolve_steps(center, velocity, t_old, t_new, delta):
    """Integer pixel steps and sub-pixel remainder of evolve_until (infinite_atmospheric_layer.py:332-342)."""
    old_px = np.round(center / delta).astype('int')
    center = center + velocity * (t_new - t_old)
    new_px = np.round(center / delta).astype('int')
    steps = new_px - old_px
    sub = center - new_px * delta
    return center, steps, sub


def phase_screen_apply(e, screen, wavelength, adjoint=False):
    """AtmosphericLayer.forward/backward, hcipy/atmosphere/atmospheric_model.py:143-151."""
    sign = -1 if adjoint else 1
    return np.asarray(e) * np.exp(sign * 1j * np.asarray(screen) / wavelength)


def von_karman_covariance(r, r0, l0):
    """phase_covariance_von_karman, hcipy/atmosphere/atmospheric_model.py:321-346."""
    from scipy.special import gamma, kv
    r = np.asarray(r, np.float64) + 1e-10
    a = (l0 / r0)**(5 / 3)
    b = gamma(11 / 6) / (2**(5 / 6) * np.pi**(8 / 3))
    c = (24 / 5 * gamma(6 / 5))**(5 / 6)
    d = (2 * np.pi * r / l0)**(5 / 6)
    e = kv(5 / 6, 2 * np.pi * r / l0)
    return a * b * c * d * e


def cn2_noise_std(cn2):
    """Standard deviation of the extrusion noise, infinite_atmospheric_layer.py:238."""
    return math.sqrt(cn2)


def von_karman_psd(grid, r0, l0):
    """hcipy/atmosphere/atmospheric_model.py:376-399 on a regular grid's points (angular frequency)."""
    x, y = grid.coords()
    u = np.hypot(x, y) + 1e-10
    u0 = 2 * np.pi / l0
    res = 0.0229 * ((u**2 + u0**2) / (2 * np.pi)**2)**(-11 / 6.) * r0**(-5 / 3)
    res[u < 1e-9] = 0
    return res


def multiscale_spectral_noise(grid, r0, l0, oversampling, rng, shift=None):
    """One realization of SpectralNoiseFactoryMultiscale (hcipy/util/spectral_noise.py:203-320) with the von
    Karman PSD, evaluated on ``grid``: the high frequencies on the FFT grid of ``grid``, the low ones on that grid
    scaled down by ``oversampling`` through a matrix Fourier transform; draws from ``rng`` in the reference's
    order (real then imaginary part of the FFT part, then of the MFT part)."""
    from .fourier import FFTPlan, mft_backward
    fft = FFTPlan(grid)
    g1 = fft.output_grid
    g2 = g1.scaled(1.0 / oversampling)
    x2, y2 = g2.coords()
    boundary = np.abs(x2).max()
    x1, y1 = g1.coords()
    c1 = np.sqrt(von_karman_psd(g1, r0, l0) / g1.weights * (2 * np.pi)**2)
    c1[np.hypot(x1, y1) < boundary] = 0
    c2 = np.sqrt(von_karman_psd(g2, r0, l0) / g2.weights * (2 * np.pi)**2)
    c2[np.hypot(x2, y2) >= boundary] = 0
    n1, n2 = g1.size, g2.size
    c1 = c1 * (rng.standard_normal(n1) + 1j * rng.standard_normal(n1))
    c2 = c2 * (rng.standard_normal(n2) + 1j * rng.standard_normal(n2))
    if shift is not None:
        # SpectralNoiseMultiscale.shift (:291-307): the ramp is the outer sum of shift[0] x and shift[1] y laid out
        # x-major (np.ix_ then ravel), multiplied onto the y-major noise as it lies in memory
        c1 = c1 * np.exp(-1j * _ix_sum(shift, g1.separated_coords))
        c2 = c2 * np.exp(-1j * _ix_sum(shift, g2.separated_coords))
    gx, gy = grid.separated_coords
    ux, uy = g2.separated_coords
    return fft.backward(c1).real + mft_backward(c2, gx, gy, ux, uy, g2.weights).real


def _ix_sum(shift, axes):
    """sum(np.ix_(*[shift[i] * axes[i]])) flattened in C order (spectral_noise.py:300-305)."""
    return (shift[0] * axes[0][:, None] + shift[1] * axes[1][None, :]).ravel()
