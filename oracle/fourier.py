"""Fourier operators of the reference, restated in float64 numpy (test infrastructure only).

Conventions follow the reference: a 2-D field is a flat vector in y-major order,
``shaped`` to ``(Ny, Nx)``; grids are ``oracle.grids.RegularGrid`` objects or
plain separated coordinate arrays.
"""
import math

import numpy as np
import scipy.fft

from .grids import make_fft_grid


# ---------------------------------------------------------------------------
# Matrix Fourier transform -- hcipy/fourier/matrix_fourier_transform.py
# ---------------------------------------------------------------------------

def mft_matrices(x, y, u, v):
    """M1 = exp(-i v (x) y) (Nv x Ny), M2 = exp(-i x (x) u) (Nx x Nu).

    matrix_fourier_transform.py:95-102.
    """
    m1 = np.exp(-1j * np.outer(v, y))
    m2 = np.exp(-1j * np.outer(x, u))
    return m1, m2


def mft_forward(e, x, y, u, v, w_in):
    """out = w_in * M1 . E . M2 (matrix_fourier_transform.py:133-176)."""
    m1, m2 = mft_matrices(x, y, u, v)
    e = np.asarray(e).reshape(len(y), len(x))
    if np.ndim(w_in) == 0:
        return (w_in * (m1 @ (e @ m2))).ravel()
    e = e * np.asarray(w_in).reshape(e.shape)
    return (m1 @ (e @ m2)).ravel()


def mft_backward(f, x, y, u, v, w_out):
    """in = w_out/(2 pi)^2 * M1^H . F . M2^H (matrix_fourier_transform.py:179-224).

    ``w_out`` is the output grid weight before the (2 pi)^2 division
    (matrix_fourier_transform.py:81).
    """
    m1, m2 = mft_matrices(x, y, u, v)
    f = np.asarray(f).reshape(len(v), len(u))
    w = np.asarray(w_out) / (2 * np.pi)**2
    if np.ndim(w) == 0:
        return (w * ((m1.conj().T @ f) @ m2.conj().T)).ravel()
    f = f * w.reshape(f.shape)
    return ((m1.conj().T @ f) @ m2.conj().T).ravel()


def mft_adjoint(f, x, y, u, v, w_in):
    """The true adjoint of ``mft_forward``: w_in * M1^H . F . M2^H."""
    m1, m2 = mft_matrices(x, y, u, v)
    f = np.asarray(f).reshape(len(v), len(u))
    out = (m1.conj().T @ f) @ m2.conj().T
    if np.ndim(w_in) == 0:
        return (w_in * out).ravel()
    return (np.asarray(w_in).reshape(out.shape) * out).ravel()


def mft1d_forward(e, x, u, w_in):
    """One-dimensional MFT, matrix_fourier_transform.py:149-151."""
    m = np.exp(-1j * np.outer(u, x))
    return m @ (np.asarray(e) * w_in)


def mft1d_backward(f, x, u, w_out):
    """matrix_fourier_transform.py:195-197 with w_out/(2 pi) (ndim 1)."""
    m = np.exp(-1j * np.outer(u, x))
    return m.conj().T @ (np.asarray(f) * (w_out / (2 * np.pi)))


def mft_cmacs(nx, ny, nu, nv):
    """Complex multiply-accumulates of the two GEMMs (matrix_fourier_transform.py:282-292)."""
    return ny * nx * nu + nv * ny * nu


# ---------------------------------------------------------------------------
# Zero-padded FFT -- hcipy/fourier/fast_fourier_transform.py:223-406
# ---------------------------------------------------------------------------

class FFTPlan(object):
    """Cutouts and phase arrays of FastFourierTransform.__init__ (fast_fourier_transform.py:223-321).

    The fftshift emulation of the reference is an algebraic identity; this
    restatement uses the exact index shifts (the ``emulate_fftshifts=False`` branch).
    """

    def __init__(self, input_grid, q=1, fov=1, shift=0):
        self.input_grid = input_grid
        self.output_grid = make_fft_grid(input_grid, q, fov, shift)
        self.internal_grid = make_fft_grid(input_grid, q, 1)
        self.shape_in = input_grid.shape
        self.shape_out = self.output_grid.shape
        self.internal_shape = self.internal_grid.shape
        if np.any(self.output_grid.dims > self.internal_grid.dims):
            raise ValueError('The amount of cropping (fov) must be smaller than 1.')

        def cut(outer, inner):
            start = tuple(int(o / 2) - int(i / 2) for o, i in zip(outer, inner))
            return tuple(slice(s, s + i) for s, i in zip(start, inner))

        self.cutout_input = cut(self.internal_shape, self.shape_in)
        self.cutout_output = cut(self.internal_shape, self.shape_out)

        # shift_input: fast_fourier_transform.py:279-297 (exact-shift branch).
        center = input_grid.zero + input_grid.delta * (input_grid.dims // 2)
        coords = self.output_grid.coords()
        s = np.exp(1j * sum(-c * k for c, k in zip(center, coords)))
        piston = np.fft.ifftshift(s.reshape(self.shape_out)).ravel()[0]
        self.shift_input = s / piston * input_grid.weights

        # shift_output: fast_fourier_transform.py:301-305.
        shift = np.ones(input_grid.ndim) * shift
        if np.allclose(shift, 0):
            self.shift_output = None
        else:
            cin = input_grid.coords()
            self.shift_output = np.exp(1j * sum(-sh * c for sh, c in zip(shift, cin)))

    def forward(self, e):
        """fast_fourier_transform.py:324-365."""
        internal = np.zeros(self.internal_shape, dtype=np.complex128)
        e = np.asarray(e, dtype=np.complex128)
        if self.shift_output is not None:
            e = e * self.shift_output
        internal[self.cutout_input] = e.reshape(self.shape_in)
        f = np.fft.fftshift(np.fft.fftn(np.fft.ifftshift(internal)))
        return f[self.cutout_output].ravel() * self.shift_input

    def backward(self, f):
        """fast_fourier_transform.py:367-406."""
        internal = np.zeros(self.internal_shape, dtype=np.complex128)
        internal[self.cutout_output] = (np.asarray(f, np.complex128) / self.shift_input).reshape(self.shape_out)
        e = np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(internal)))
        res = e[self.cutout_input].ravel()
        if self.shift_output is not None:
            res = res / self.shift_output
        return res


# ---------------------------------------------------------------------------
# Chirp-Z transform -- hcipy/fourier/chirp_z_transform.py:51-105
# ---------------------------------------------------------------------------

def czt(x, m, w, a):
    """Bluestein evaluation of X_k = sum_n x_n (a w^-k)^-n along the last axis.

    chirp_z_transform.py:51-71 (kernel) and :93-105 (call).
    """
    x = np.asarray(x, dtype=np.complex128)
    n = x.shape[-1]
    w = complex(w)
    a = complex(a)
    k = np.arange(max(m, n))
    wk2 = w**(k**2 / 2)
    nfft = scipy.fft.next_fast_len(n + m - 1)
    awk2 = a**-k[:n] * wk2[:n]
    fwk2 = np.fft.fft(1 / np.hstack((wk2[n - 1:0:-1], wk2[:m])), n=nfft)
    y = np.fft.ifft(np.fft.fft(x * awk2, n=nfft) * fwk2)
    return y[..., n - 1:n + m - 1] * wk2[:m]


def czt_direct(x, m, w, a):
    """Direct O(nm) sum of the same transform, for cross-checks on small sizes."""
    x = np.asarray(x, dtype=np.complex128)
    n = x.shape[-1]
    z = complex(a) * complex(w)**(-np.arange(m))
    mat = z[:, None]**(-np.arange(n)[None, :])
    return x @ mat.T


# ---------------------------------------------------------------------------
# Zoom FFT -- hcipy/fourier/zoom_fast_fourier_transform.py:43-119
# ---------------------------------------------------------------------------

def zoomfft_forward(e, input_grid, output_grid):
    """zoom_fast_fourier_transform.py:69-93 (2-D)."""
    f = (np.asarray(e) * input_grid.weights).reshape(input_grid.shape)
    for axis in (0, 1):
        n, m = input_grid.dims[axis], output_grid.dims[axis]
        w = np.exp(-1j * output_grid.delta[axis] * input_grid.delta[axis])
        a = np.exp(1j * output_grid.zero[axis] * input_grid.delta[axis])
        shift = np.exp(-1j * output_grid.axis(axis) * input_grid.zero[axis])
        f = np.moveaxis(f, 1 - axis, -1)
        f = czt(f, m, w, a) * shift
        f = np.moveaxis(f, -1, 1 - axis)
    return f.ravel()


def zoomfft_backward(f, input_grid, output_grid):
    """zoom_fast_fourier_transform.py:95-119 (2-D)."""
    g = (np.asarray(f) * output_grid.weights / (2 * math.pi)**2).reshape(output_grid.shape)
    for axis in (0, 1):
        n, m = output_grid.dims[axis], input_grid.dims[axis]
        w = np.exp(1j * input_grid.delta[axis] * output_grid.delta[axis])
        a = np.exp(-1j * input_grid.zero[axis] * output_grid.delta[axis])
        shift = np.exp(1j * input_grid.axis(axis) * output_grid.zero[axis])
        g = np.moveaxis(g, 1 - axis, -1)
        g = czt(g, m, w, a) * shift
        g = np.moveaxis(g, -1, 1 - axis)
    return g.ravel()


# ---------------------------------------------------------------------------
# Fourier filter and angular-spectrum transfer function
# ---------------------------------------------------------------------------

class FourierFilterPlan(object):
    """hcipy/fourier/fourier_operations.py:28-151 for a scalar transfer function."""

    def __init__(self, input_grid, tf_centered, q=1):
        fft = FFTPlan(input_grid, q)
        self.input_grid = input_grid
        self.internal_grid = fft.output_grid
        self.cutout = fft.cutout_input
        self.shape_in = input_grid.shape
        # fourier_operations.py:47-48: ifftshift of the shaped transfer function.
        self.tf = np.fft.ifftshift(np.asarray(tf_centered).reshape(self.internal_grid.shape))

    def apply(self, e, adjoint=False):
        f = np.zeros(self.internal_grid.shape, dtype=np.complex128)
        f[self.cutout] = np.asarray(e).reshape(self.shape_in)
        f = np.fft.fftn(f)
        f = f * (self.tf.conj() if adjoint else self.tf)
        f = np.fft.ifftn(f)
        return f[self.cutout].ravel()


def supersampled_mean(func, grid, oversampling=2):
    """evaluate_supersampled for a separated grid with statistic 'mean' (hcipy/field/util.py:655-692)."""
    axes = grid.separated_coords
    deltas = []
    for x in axes:
        d = (x[2:] - x[:-2]) / 2.
        deltas.append(np.concatenate(([x[1] - x[0]], d, [x[-1] - x[-2]])))
    # make_uniform_grid(oversampling, 1): dither offsets in units of the local spacing.
    dz = 1.0 / oversampling
    offsets = -0.5 + dz / 2 + dz * np.arange(oversampling)
    total = 0
    count = 0
    for oy in offsets:
        for ox in offsets:
            xs = axes[0] + ox * deltas[0]
            ys = axes[1] + oy * deltas[1]
            xx, yy = np.meshgrid(xs, ys, indexing='xy')
            total = total + func(xx.ravel(), yy.ravel())
            count += 1
    return total / count


def asp_transfer_function(internal_grid, wavelength, distance, refractive_index=1, oversampling=2):
    """Native transfer-function branch, hcipy/propagation/angular_spectrum.py:137-166."""
    k = 2 * np.pi / wavelength * refractive_index

    def tf(kx, ky):
        k_squared = kx**2 + ky**2
        k_z = np.sqrt(k**2 - k_squared + 0j)
        return np.exp(1j * k_z * distance)

    return supersampled_mean(tf, internal_grid, oversampling)


def asp_uses_impulse_branch(input_grid, wavelength, distance):
    """angular_spectrum.py:139-143."""
    l_max = np.max(input_grid.dims * input_grid.delta)
    return bool(np.any(input_grid.delta < wavelength * abs(distance) / l_max))


# ---------------------------------------------------------------------------
# Fresnel propagation -- hcipy/propagation/fresnel.py:45-80
# ---------------------------------------------------------------------------

def fresnel_uses_impulse_branch(input_grid, wavelength, distance):
    """fresnel.py:47-50 (the same sampling test as the angular-spectrum propagator)."""
    return asp_uses_impulse_branch(input_grid, wavelength, distance)


def fresnel_transfer_function(internal_grid, wavelength, distance, refractive_index=1, oversampling=2):
    """Native branch, fresnel.py:69-80: exp(i k d) exp(-i d/(2k) (kx^2 + ky^2)), supersampled."""
    k = 2 * np.pi / wavelength * refractive_index
    phase_factor = np.exp(1j * k * distance)

    def tf(kx, ky):
        return phase_factor * np.exp(-0.5j * distance / k * (kx * kx + ky * ky))

    return supersampled_mean(tf, internal_grid, oversampling)


def fresnel_impulse_transfer_function(internal_grid, wavelength, distance, refractive_index=1, oversampling=2):
    """Impulse-response branch, fresnel.py:51-67: the impulse response exp(i k d)/(i lambda d) exp(i k/(2d) r^2),
    supersampled on the spatial grid of the Fourier grid, transformed by the (unpadded) FFT."""
    from .grids import make_fft_grid
    k = 2 * np.pi / wavelength * refractive_index
    enlarged = make_fft_grid(internal_grid)
    phase_factor = np.exp(1j * k * distance) / (1j * wavelength * distance)

    def ir(x, y):
        return phase_factor * np.exp(0.5j * k / distance * (x * x + y * y))

    return FFTPlan(enlarged).forward(supersampled_mean(ir, enlarged, oversampling))
