"""Atmospheric layers (hcipy/atmosphere) with the per-frame work on the device.

``InfiniteAtmosphericLayer`` follows hcipy/atmosphere/infinite_atmospheric_layer.py: the same stencils
(including the random far pixel of each column, drawn from the layer's generator first, :111-140), the same
von Karman covariances and autoregressive matrices A = C_xz C_zz^-1 and B from the SVD of C_xx - A C_zx
(:142-202), and the same extrusion and time stepping (:216-364).  Plan-time work (covariances, Cholesky,
SVD) runs on the host in float64 as in the reference; every frame runs on the GPU:

* the screen is a ring buffer with a spare row and column, so an extrusion moves an offset and writes one row
  or column into the spare slice (``hx_atmosphere_extrude``: A . stencil + B . noise, the stencil gathered by
  the same launch) instead of copying the screen; a ``MultiLayerAtmosphere`` frame extrudes step k of all its
  layers in one launch (``hx_atmosphere_extrude_layers``);
* the extrusion noise is drawn on the host from the layer's numpy Generator with the reference's call,
  ``rng.normal(0, sqrt(Cn^2), size=B.shape[1])``, one draw per step in the reference's order, so a layer seeded
  like the reference's extrudes the same rows;
* the quintic sub-pixel shift (hcipy/_math/subpixel_shift.py) reads the ring and writes the shifted screen
  (``hx_atmosphere_shift``); a ``MultiLayerAtmosphere`` frame shifts all its layers and sums their screens in
  one pass (``hx_atmosphere_shift_layers``);
* ``forward``/``backward`` multiply by exp(+-i screen / lambda) in one kernel (``hx_phase_apply``).

The initial screen is the reference's: multi-scale spectral noise at oversampling 16
(``SpectralNoiseFactoryMultiscale``, hcipy/util/spectral_noise.py:203-320), its random draws taken from the layer's
generator in the reference's order after the stencil draws, and evaluated with this package's own padded FFT and
matrix Fourier transform on the device in float64 (construction time only), so a layer seeded like the reference's
starts from the reference's screen and extrudes the reference's rows.  ``initial_screen`` sets it explicitly.
"""
import copy
import math

import numpy as np
import torch

from . import _lib
from .field import Field, as_tensor
from .kernels import apply_phase
from .optics import OpticalElement


# ---- turbulence statistics (hcipy/atmosphere/atmospheric_model.py:321-420) -------------------------------

def Cn_squared_from_fried_parameter(r0, wavelength=500e-9):  # noqa: N802
    k = 2 * np.pi / wavelength
    return r0**(-5. / 3) / (0.423 * k**2)


def fried_parameter_from_Cn_squared(Cn_squared, wavelength=500e-9):  # noqa: N802
    k = 2 * np.pi / wavelength
    return (0.423 * Cn_squared * k**2)**(-3. / 5)


def von_karman_covariance(r, r0, L0):  # noqa: N803
    """Phase covariance of von Karman turbulence at separations r (atmospheric_model.py:321-346)."""
    from scipy.special import gamma, kv
    r = np.asarray(r, np.float64) + 1e-10
    a = (L0 / r0)**(5 / 3)
    b = gamma(11 / 6) / (2**(5 / 6) * np.pi**(8 / 3))
    c = (24 / 5 * gamma(6 / 5))**(5 / 6)
    d = (2 * np.pi * r / L0)**(5 / 6)
    e = kv(5 / 6, 2 * np.pi * r / L0)
    return a * b * c * d * e


def quintic_weights(shift):
    """7-tap quintic B-spline weights of a shift in [-0.5, 0.5] pixels (subpixel_shift.py:7-35)."""
    f = abs(shift)
    b = np.empty(6)
    for i, offset in enumerate((2.0 + f, 1.0 + f, f, 1.0 - f, 2.0 - f, 3.0 - f)):
        acc, x = 0.0, offset + 3.0
        for c in (1.0, -6.0, 15.0, -20.0, 15.0, -6.0, 1.0):
            if x > 0.0:
                acc += c * x**5
            x -= 1.0
        b[i] = acc / 120.0
    if shift >= 0:
        return np.array([0.0, b[0], b[1], b[2], b[3], b[4], b[5]])
    return np.array([b[5], b[4], b[3], b[2], b[1], b[0], 0.0])


def power_spectral_density_von_karman(r0, L0):  # noqa: N803
    """The von Karman phase PSD as a function of a grid of angular frequencies (atmospheric_model.py:376-399):
    0.0229 ((u^2 + u0^2) / (2 pi)^2)^(-11/6) r0^(-5/3), u0 = 2 pi / L0, zero at the origin.  Returns float64
    values on the host, one per grid point."""
    def func(grid):
        x, y = (np.asarray(c, np.float64) for c in grid.points_list())
        u = np.hypot(x, y) + 1e-10
        u0 = 2 * np.pi / L0
        res = 0.0229 * ((u**2 + u0**2) / (2 * np.pi)**2)**(-11 / 6.) * r0**(-5 / 3)
        res[u < 1e-9] = 0
        return res
    return func


class SpectralNoiseFactoryMultiscale(object):
    """Spectral noise from two Fourier transforms (hcipy/util/spectral_noise.py:203-264): the PSD's high
    frequencies on the FFT grid of ``output_grid`` (padded FFT), the low ones on that grid scaled down by
    ``oversampling`` (matrix Fourier transform), split at the largest frequency of the fine grid.  The amplitudes
    are host float64 arrays; a realization lives on the device in complex128."""

    def __init__(self, psd, output_grid, oversampling):
        from .fft import FastFourierTransform
        from .fourier import MatrixFourierTransform
        self.psd = psd
        self.output_grid = output_grid
        self.oversampling = oversampling
        self.fourier_1 = FastFourierTransform(output_grid)
        self.input_grid_1 = self.fourier_1.output_grid
        self.input_grid_2 = self.input_grid_1.scaled(1.0 / oversampling)
        self.fourier_2 = MatrixFourierTransform(output_grid, self.input_grid_2)
        boundary = np.abs(np.asarray(self.input_grid_2.points_list()[0], np.float64)).max()
        r1 = np.hypot(*(np.asarray(c, np.float64) for c in self.input_grid_1.points_list()))
        r2 = np.hypot(*(np.asarray(c, np.float64) for c in self.input_grid_2.points_list()))
        nd = self.input_grid_1.ndim
        w1 = float(np.asarray(self.input_grid_1.weights).ravel()[0])
        w2 = float(np.asarray(self.input_grid_2.weights).ravel()[0])
        # (2 pi)^ndim converts the PSD per Hertz to per radian
        self.C_1 = np.sqrt(psd(self.input_grid_1) / w1 * (2 * np.pi)**nd)
        self.C_1[r1 < boundary] = 0
        self.C_2 = np.sqrt(psd(self.input_grid_2) / w2 * (2 * np.pi)**nd)
        self.C_2[r2 >= boundary] = 0

    def make_random(self, seed=None):
        """One realization (spectral_noise.py:266-289): complex normal draws from ``numpy.random.default_rng(seed)``
        in the reference's order, real then imaginary part of the fine grid, then of the coarse grid."""
        rng = np.random.default_rng(seed)
        n1, n2 = self.input_grid_1.size, self.input_grid_2.size
        c1 = self.C_1 * (rng.standard_normal(n1) + 1j * rng.standard_normal(n1))
        c2 = self.C_2 * (rng.standard_normal(n2) + 1j * rng.standard_normal(n2))
        return SpectralNoiseMultiscale(self, c1, c2)


class SpectralNoiseMultiscale(object):
    """A realization of multi-scale spectral noise (spectral_noise.py:266-320) with its two spectra on the
    device."""

    def __init__(self, factory, C_1, C_2):  # noqa: N803
        self.factory = factory
        dev = torch.device('cuda')
        self.C_1 = torch.as_tensor(np.asarray(C_1, np.complex128), device=dev)
        self.C_2 = torch.as_tensor(np.asarray(C_2, np.complex128), device=dev)

    def copy(self):
        out = SpectralNoiseMultiscale.__new__(SpectralNoiseMultiscale)
        out.factory, out.C_1, out.C_2 = self.factory, self.C_1.clone(), self.C_2.clone()
        return out

    def shift(self, shift):
        """In-place shift by ``shift`` (grid units) as a phase ramp on both spectra (spectral_noise.py:291-307).
        The reference forms the ramp as an outer sum over (x, y) flattened x-major and multiplies it onto the
        y-major spectrum as it lies in memory; the same layout is kept so that shifted screens match."""
        for name, grid in (('C_1', self.factory.input_grid_1), ('C_2', self.factory.input_grid_2)):
            xs, ys = (np.asarray(c, np.float64) for c in grid.separated_coords)
            ramp = np.exp(-1j * (shift[0] * xs[:, None] + shift[1] * ys[None, :]).ravel())
            setattr(self, name, getattr(self, name) * torch.as_tensor(ramp, device=self.C_1.device))

    def shifted(self, shift):
        out = self.copy()
        out.shift(shift)
        return out

    def __call__(self):
        """The noise on the factory's output grid (spectral_noise.py:309-320), float64 on the device."""
        f = self.factory
        ps = f.fourier_1.backward(Field(self.C_1, f.input_grid_1)).data.real
        ps = ps + f.fourier_2.backward(Field(self.C_2, f.input_grid_2)).data.real
        return Field(ps.contiguous(), f.output_grid)


def von_karman_screen(nx, ny, delta, Cn_squared, L0, rng, pad=2):  # noqa: N803
    """An FFT phase screen (radians at wavelength 1 m) of pad times the extent, cropped to ny x nx."""
    n = pad * max(nx, ny)
    d = float(np.max(delta))
    k = 2 * np.pi * np.fft.fftfreq(n, d)
    kx, ky = np.meshgrid(k, k)
    k0 = 2 * np.pi / L0 if np.isfinite(L0) else 0.0
    r0 = fried_parameter_from_Cn_squared(Cn_squared, 1.0)
    # 0.023 r0^-5/3 f^-11/3 per (cycle/m)^2, written for angular frequency k = 2 pi f
    psd = 0.023 * (2 * np.pi)**(5 / 3) * r0**(-5 / 3) * (kx**2 + ky**2 + k0**2)**(-11 / 6)
    psd[0, 0] = 0.0
    dk = 2 * np.pi / (n * d)
    c = np.sqrt(psd) * dk * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    screen = np.real(np.fft.ifft2(c)) * n * n
    return screen[:ny, :nx].copy()


def make_stencils(nx, ny, stencil_length, rng):
    """Flat indices of the bottom and left stencils: the first ``stencil_length`` rows (columns) plus one pixel
    per column (row) at a geometric distance, drawn from ``rng`` in the reference's order
    (infinite_atmospheric_layer.py:111-140)."""
    st = np.zeros((ny, nx), bool)
    st[:stencil_length, :] = True
    for i, n in enumerate(rng.geometric(0.5, nx)):
        st[(n + stencil_length - 1) % ny, i] = True
    bottom = np.where(st.ravel())[0]
    st = np.zeros((ny, nx), bool)
    st[:, :stencil_length] = True
    for i, n in enumerate(rng.geometric(0.5, ny)):
        st[i, (n + stencil_length - 1) % nx] = True
    left = np.where(st.ravel())[0]
    return bottom, left


def ar_matrices(grid, stencil_idx, where, L0):  # noqa: N803
    """Autoregressive matrices of one extrusion direction for unit Cn^2 (infinite_atmospheric_layer.py:142-202):
    the von Karman covariance of stencil and new slice, A = C_xz C_zz^-1 (Cholesky), B = U sqrt(S) from the SVD
    of C_xx - A C_zx."""
    from scipy import linalg
    xs, ys = (np.asarray(c, np.float64) for c in grid.separated_coords)
    d = np.asarray(grid.delta, np.float64)
    xx, yy = np.meshgrid(xs, ys)
    px, py = xx.ravel(), yy.ravel()
    if where == 'bottom':
        new_x, new_y = xs, np.full(xs.size, ys[0] - d[1])
    else:
        new_x, new_y = np.full(ys.size, xs[0] - d[0]), ys
    x = np.concatenate((px[stencil_idx], new_x))
    y = np.concatenate((py[stencil_idx], new_y))
    sep = np.hypot(x[None, :] - x[:, None], y[None, :] - y[:, None])
    cov = von_karman_covariance(sep, fried_parameter_from_Cn_squared(1, 1), L0)
    n = stencil_idx.size
    cov_zz, cov_xz, cov_zx, cov_xx = cov[:n, :n], cov[n:, :n], cov[:n, n:], cov[n:, n:]
    cf = linalg.cho_factor(cov_zz)
    a = cov_xz.dot(linalg.cho_solve(cf, np.eye(n)))
    u, sv, _ = np.linalg.svd(cov_xx - a.dot(cov_zx))
    b = u * np.sqrt(sv[:new_x.size])
    return a, b


def subpixel_shift(img, row_shift, col_shift):
    """Shift an image (ny, nx) by fractions of a pixel with the quintic B-spline (subpixel_shift.py:306-343)."""
    if not (-0.5 <= row_shift <= 0.5) or not (-0.5 <= col_shift <= 0.5):
        raise ValueError('row_shift and col_shift must be in [-0.5, 0.5]')
    t = as_tensor(img).contiguous()
    if t.dtype not in (torch.float32, torch.float64):
        t = t.to(torch.float64)
    ny, nx = t.shape[-2:]
    out = torch.empty_like(t)
    tr = np.ascontiguousarray(quintic_weights(col_shift))
    tc = np.ascontiguousarray(quintic_weights(row_shift))
    P = _lib.ctypes.POINTER(_lib.ctypes.c_double)
    rc = _lib.lib().hx_atmosphere_shift(_lib.dptr(t), int(ny), int(nx), int(ny), int(nx), 0, 0, tr.ctypes.data_as(P),
                                        tc.ctypes.data_as(P), _lib.dptr(out), _lib.dtype_code(t.dtype),
                                        _lib.stream_handle())
    _lib.check(rc, 'hx_atmosphere_shift')
    return out


# ---- layers ---------------------------------------------------------------------------------------------

class _NoiseStage(object):
    """Noise rows to the device without stalling the host: the rows go through one of two pinned host buffers
    with an asynchronous copy on the current stream, so evolving a layer does not wait for the GPU work queued
    before it (a copy from pageable memory would); a buffer is refilled only after the event recorded behind its
    previous copy."""

    def __init__(self, dtype):
        self.dtype = dtype
        self.slot = 1
        self.host, self.event = [None, None], [None, None]
        self.dev = None

    def upload(self, draws):
        """(len(draws), width) device tensor of the rows, zero-padded to the longest."""
        width = max(x.size for x in draws)
        need = len(draws) * width
        self.slot = slot = (self.slot + 1) % 2
        if self.event[slot] is not None:
            self.event[slot].synchronize()
        buf = self.host[slot]
        if buf is None or buf.numel() < need:
            buf = self.host[slot] = torch.empty(need, dtype=self.dtype, pin_memory=True)
        if self.dev is None or self.dev.numel() < need:
            self.dev = torch.empty(need, dtype=self.dtype, device='cuda')
        host = buf[:need].numpy().reshape(len(draws), width)
        host[...] = 0
        for i, x in enumerate(draws):
            host[i, :x.size] = x
        dev = self.dev[:need]
        dev.copy_(buf[:need], non_blocking=True)
        if self.event[slot] is None:
            self.event[slot] = torch.cuda.Event()
        self.event[slot].record()
        return dev.view(len(draws), width)


class AtmosphericLayer(OpticalElement):
    """Base of the atmospheric layers (atmospheric_model.py:10-151): E exp(+-i phase_for(lambda))."""

    def __init__(self, input_grid, Cn_squared, L0=np.inf, velocity=0, height=0):  # noqa: N803
        self.input_grid = input_grid
        self._Cn_squared = Cn_squared
        self._L0 = L0
        self.velocity = velocity
        self.height = height
        self._t = 0
        self._version = 0  # bumped whenever the device screen changes (combined screens key on it)

    @property
    def t(self):
        return self._t

    @t.setter
    def t(self, t):
        self.evolve_until(t)

    @property
    def velocity(self):
        return self._velocity

    @velocity.setter
    def velocity(self, velocity):
        self._velocity = np.array([velocity, 0.0]) if np.isscalar(velocity) else np.array(velocity, np.float64)

    @property
    def outer_scale(self):
        return self._L0

    @outer_scale.setter
    def outer_scale(self, L0):  # noqa: N803
        self._L0 = L0

    @property
    def L0(self):  # noqa: N802
        return self.outer_scale

    @L0.setter
    def L0(self, L0):  # noqa: N802, N803
        self.outer_scale = L0

    @property
    def output_grid(self):
        return self.input_grid

    def _screen_tensor(self):
        raise NotImplementedError()

    def phase_for(self, wavelength):
        return Field(self._screen_tensor() / wavelength, self.input_grid)

    def _apply(self, wf, sign):
        e = as_tensor(wf.electric_field)
        s = self._screen_tensor()
        if torch.is_grad_enabled() and e.requires_grad:
            from .autograd import phase_apply
            out = phase_apply(e, s, sign / wf.wavelength)
        else:
            out = apply_phase(e, s, sign / wf.wavelength)
        return wf._carry(Field(out, wf.electric_field.grid))

    def forward(self, wf):
        return self._apply(wf, 1.0)

    def backward(self, wf):
        return self._apply(wf, -1.0)

    def _pure_phase_screen(self):
        """The screen s (radians at 1 m) whose forward is exp(i s / wavelength): a consumer may fuse the phase."""
        return self._screen_tensor()


_WHERE = {'bottom': 0, 'top': 1, 'left': 2, 'right': 3}


class InfiniteAtmosphericLayer(AtmosphericLayer):
    """An infinitely extendable layer (Assemat et al. 2006), infinite_atmospheric_layer.py:14-390.

    Extra arguments: ``dtype`` of the device screen and AR matrices (float64 as the reference, or float32 to
    halve the bytes of every extrusion), ``initial_screen`` (ny x nx, radians at 1 m) instead of the generated
    one.
    """

    def __init__(self, input_grid, Cn_squared, L0=np.inf, velocity=0, height=0, stencil_length=2,  # noqa: N803
                 use_interpolation=True, seed=None, dtype=torch.float64, initial_screen=None):
        self._initialized = False
        AtmosphericLayer.__init__(self, input_grid, Cn_squared, L0, velocity, height)
        if not getattr(input_grid, 'is_regular', False):
            raise ValueError('Input grid must be regularly spaced')
        if input_grid.ndim != 2:
            raise ValueError('Input grid must be two-dimensional.')
        self.stencil_length = stencil_length
        self.use_interpolation = use_interpolation
        self.dtype = dtype
        self.rng = np.random.default_rng(seed)
        self._initial_screen = None if initial_screen is None else np.asarray(initial_screen, np.float64)
        self.nx, self.ny = (int(d) for d in input_grid.dims)
        self._delta = np.asarray(input_grid.delta, np.float64)
        self._make_stencils()
        self._make_ab_matrices()
        self._original_rng = self.rng
        self.reset()
        self._initialized = True

    # -- plan-time matrices (host, float64) --------------------------------------------------------------
    def _make_stencils(self):
        self.stencil_bottom_idx, self.stencil_left_idx = make_stencils(self.nx, self.ny, self.stencil_length, self.rng)
        self.stencil_bottom = np.zeros(self.nx * self.ny, bool)
        self.stencil_bottom[self.stencil_bottom_idx] = True
        self.stencil_left = np.zeros(self.nx * self.ny, bool)
        self.stencil_left[self.stencil_left_idx] = True

    def _make_ab_matrices(self):
        g = self.input_grid
        self.A_vertical, self.B_vertical = ar_matrices(g, self.stencil_bottom_idx, 'bottom', self._L0)
        self.A_horizontal, self.B_horizontal = ar_matrices(g, self.stencil_left_idx, 'left', self._L0)
        self._upload_matrices()

    def _upload_matrices(self):
        dev, dt = torch.device('cuda'), self.dtype
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dt)  # noqa: E731
        self._dev = {
            'A_v': t(self.A_vertical), 'B_v': t(self.B_vertical),
            'A_h': t(self.A_horizontal), 'B_h': t(self.B_horizontal),
            'idx_v': torch.from_numpy(self.stencil_bottom_idx.astype(np.int64)).to(dev),
            'idx_h': torch.from_numpy(self.stencil_left_idx.astype(np.int64)).to(dev),
        }
        self._work = torch.empty(max(self.stencil_bottom_idx.size, self.stencil_left_idx.size), dtype=dt, device=dev)

    # -- state ---------------------------------------------------------------------------------------------
    def reset(self, make_independent_realization=False):
        """infinite_atmospheric_layer.py:276-303."""
        if make_independent_realization:
            self._original_rng = copy.deepcopy(self.rng)
        else:
            self.rng = copy.deepcopy(self._original_rng)
        if self._initial_screen is not None:
            screen = torch.from_numpy(np.ascontiguousarray(self._initial_screen.reshape(self.ny, self.nx)))
        else:
            screen = self._reference_initial_screen()
        screen = screen.to(device='cuda', dtype=self.dtype).reshape(self.ny, self.nx)
        if getattr(self, '_ring', None) is not None and self._ring.shape == (self.ny + 1, self.nx + 1):
            # in place: a captured CUDA graph that reads these buffers stays valid across resets
            self._ring[:self.ny, :self.nx].copy_(screen)
            self._shifted.copy_(screen)
        else:
            # the ring holds a spare row and column (outside the screen) that the next extrusion writes
            self._ring = torch.zeros((self.ny + 1, self.nx + 1), dtype=self.dtype, device='cuda')
            self._ring[:self.ny, :self.nx].copy_(screen)
            self._shifted = screen.clone()
        self._row0 = 0
        self._col0 = 0
        self._version += 1
        self.center = np.zeros(2)
        self._t = 0

    def _reference_initial_screen(self):
        """The reference's initial screen (infinite_atmospheric_layer.py:204-214): the phase at a wavelength of 1 m
        of a finite layer with oversampling 16, i.e. multi-scale spectral noise with the von Karman PSD of this
        layer's turbulence, drawn from the layer's generator (which then continues with the extrusion noise)."""
        psd = power_spectral_density_von_karman(fried_parameter_from_Cn_squared(self._Cn_squared, 1), self._L0)
        factory = SpectralNoiseFactoryMultiscale(psd, self.input_grid, 16)
        return factory.make_random(self.rng)().data

    @property
    def Cn_squared(self):  # noqa: N802
        return self._Cn_squared

    @Cn_squared.setter
    def Cn_squared(self, Cn_squared):  # noqa: N802, N803
        self._Cn_squared = Cn_squared

    @property
    def outer_scale(self):
        return self._L0

    @outer_scale.setter
    def outer_scale(self, L0):  # noqa: N803
        self._L0 = L0
        if self._initialized:
            self._make_ab_matrices()

    # -- time stepping -------------------------------------------------------------------------------------
    def _step_matrices(self, where):
        d = self._dev
        if _WHERE[where] <= 1:
            return d['A_v'], d['B_v'], d['idx_v']
        return d['A_h'], d['B_h'], d['idx_h']

    def _extrusion(self, where, noise):
        """The ``hx_extrusion`` record of one step from the current offsets."""
        A, B, idx = self._step_matrices(where)
        return _lib.Extrusion(_lib.dptr(self._ring), _lib.dptr(idx), _lib.dptr(A), _lib.dptr(B), _lib.dptr(noise),
                              self.ny, self.nx, self._row0, self._col0, _WHERE[where], int(idx.numel()),
                              int(B.shape[1]))

    def _moved(self, where):
        """The offsets after an extrusion (the spare slice becomes the new edge)."""
        w = _WHERE[where]
        if w == 0:
            self._row0 = (self._row0 - 1) % (self.ny + 1)
        elif w == 1:
            self._row0 = (self._row0 + 1) % (self.ny + 1)
        elif w == 2:
            self._col0 = (self._col0 - 1) % (self.nx + 1)
        else:
            self._col0 = (self._col0 + 1) % (self.nx + 1)
        self._version += 1

    def _extrude(self, where, noise):
        A, B, idx = self._step_matrices(where)
        rc = _lib.lib().hx_atmosphere_extrude(_lib.dptr(self._ring), self.ny, self.nx, self._row0, self._col0,
                                              _WHERE[where], _lib.dptr(idx), int(idx.numel()), _lib.dptr(A),
                                              _lib.dptr(B), int(B.shape[1]), _lib.dptr(noise),
                                              _lib.dtype_code(self.dtype), _lib.stream_handle())
        _lib.check(rc, 'hx_atmosphere_extrude')
        self._moved(where)

    def _advance(self, t):
        """The host part of ``evolve_until`` (infinite_atmospheric_layer.py:305-364): moves the layer's clock and
        centre, draws the steps' noise from the generator in the reference's order and returns (steps, noise rows,
        row taps, column taps) for the device."""
        if t < self._t:
            raise ValueError('Backwards temporal evolution is not allowed.')
        delta = self._delta
        old_center = np.round(self.center / delta).astype('int')
        self.center = self.center + self.velocity * (t - self._t)
        new_center = np.round(self.center / delta).astype('int')
        self._t = t
        steps = new_center - old_center
        sub = self.center - new_center * delta
        plan = (['left' if steps[0] < 0 else 'right'] * abs(int(steps[0])) +
                ['bottom' if steps[1] < 0 else 'top'] * abs(int(steps[1])))
        std = math.sqrt(self._Cn_squared)
        draws = [self.rng.normal(0, std, size=(self.B_vertical if _WHERE[w] <= 1 else self.B_horizontal).shape[1])
                 for w in plan]
        if self.use_interpolation:
            shift = sub / delta  # [x_px, y_px]
            taps_row = quintic_weights(shift[0])  # along x
            taps_col = quintic_weights(shift[1])  # along y
        else:
            taps_row = taps_col = np.array([0, 0, 0, 1.0, 0, 0, 0])
        return plan, draws, taps_row, taps_col

    def evolve_until(self, t):
        """infinite_atmospheric_layer.py:305-364."""
        if t is None:
            self.reset()
            return
        plan, draws, taps_row, taps_col = self._advance(t)
        if plan:
            noise = self._upload_noise(draws)
            for i, w in enumerate(plan):
                self._extrude(w, noise[i])
        self._shift(taps_row, taps_col)

    def _upload_noise(self, draws):
        """The steps' noise rows on the device (len(draws) x width, zero-padded), without stalling the host."""
        if getattr(self, '_noise', None) is None:
            self._noise = _NoiseStage(self.dtype)
        return self._noise.upload(draws)

    def _shift(self, taps_row, taps_col):
        tr = np.ascontiguousarray(taps_row, np.float64)
        tc = np.ascontiguousarray(taps_col, np.float64)
        P = _lib.ctypes.POINTER(_lib.ctypes.c_double)
        rc = _lib.lib().hx_atmosphere_shift(_lib.dptr(self._ring), self.ny + 1, self.nx + 1, self.ny, self.nx,
                                            self._row0, self._col0, tr.ctypes.data_as(P), tc.ctypes.data_as(P),
                                            _lib.dptr(self._shifted), _lib.dtype_code(self.dtype),
                                            _lib.stream_handle())
        _lib.check(rc, 'hx_atmosphere_shift')
        self._version += 1

    # -- screens -------------------------------------------------------------------------------------------
    @property
    def achromatic_screen(self):
        """The unshifted screen (logical order), radians at a wavelength of 1 m."""
        taps = np.array([0, 0, 0, 1.0, 0, 0, 0])
        out = torch.empty_like(self._shifted)
        P = _lib.ctypes.POINTER(_lib.ctypes.c_double)
        rc = _lib.lib().hx_atmosphere_shift(_lib.dptr(self._ring), self.ny + 1, self.nx + 1, self.ny, self.nx,
                                            self._row0, self._col0, taps.ctypes.data_as(P), taps.ctypes.data_as(P),
                                            _lib.dptr(out), _lib.dtype_code(self.dtype), _lib.stream_handle())
        _lib.check(rc, 'hx_atmosphere_shift')
        return Field(out.reshape(-1), self.input_grid)

    def _screen_tensor(self):
        return self._shifted.reshape(-1)


class MultiLayerAtmosphere(OpticalElement):
    """Layers applied in sequence (atmospheric_model.py:153-310).

    Without scintillation the reference applies the layers one after the other, sorted by height (:185-212,
    :300-308); with no propagation between them the product of their phase factors is the phase factor of the
    summed screens, so ``forward``/``backward`` sum the layers' screens once (``hx_atmosphere_combine``, into a
    buffer that keeps its address) and apply one phase kernel.  ``evolve_until`` refreshes the sum, so a CUDA
    graph that captured ``forward`` replays with the current screens; after evolving a layer on its own, call
    ``combined_screen()`` before replaying such a graph.

    With ``scintillation=True`` the layers are applied from the highest down with a Fresnel propagation over the
    height difference between consecutive layers and from the lowest layer to the ground (:191-210).
    """

    def __init__(self, layers, scintillation=False):
        self.layers = list(layers)
        self._scintillation = bool(scintillation)
        self._t = 0
        self._combined = None
        self._combined_key = None
        self._elements = None

    @property
    def scintillation(self):
        return self._scintillation

    @scintillation.setter
    def scintillation(self, scintillation):
        self._scintillation = bool(scintillation)
        self._elements = None

    def calculate_propagators(self):
        """The element sequence of the scintillating form (atmospheric_model.py:185-212)."""
        from .propagation import FresnelPropagator
        heights = np.array([layer.height for layer in self.layers], np.float64)
        order = np.argsort(-heights, kind='stable')
        h = heights[order]
        grid = self.layers[0].input_grid
        elements = []
        for i, j in enumerate(order):
            elements.append(self.layers[j])
            if i < len(order) - 1:
                elements.append(FresnelPropagator(grid, h[i] - h[i + 1]))
        if h[-1] > 0:
            elements.append(FresnelPropagator(grid, h[-1]))
        self._elements = elements
        return elements

    def evolve_until(self, t):
        """Every layer to time t (atmospheric_model.py:237-246).  When the layers are infinite layers of one grid
        and screen dtype (up to 8), the frame runs as one batch: the host plans and noise draws of all layers
        (each layer's generator in the reference's order), one upload of the noise, one extrusion launch per step
        index (step k of every layer that moves k or more pixels), then one pass that shifts every layer's screen
        and writes their sum."""
        if t is not None and self._batchable():
            self._evolve_batched(t)
        else:
            for layer in self.layers:
                layer.evolve_until(t)
        self._t = t
        self.combined_screen()

    def _batchable(self):
        layers = self.layers
        if not layers or len(layers) > 8:
            return False
        if any(type(layer).evolve_until is not InfiniteAtmosphericLayer.evolve_until for layer in layers):
            return False
        first = layers[0]
        return all(layer.nx == first.nx and layer.ny == first.ny and layer.dtype == first.dtype for layer in layers)

    def _evolve_batched(self, t):
        layers = self.layers
        first = layers[0]
        plans = [layer._advance(t) for layer in layers]
        draws = [d for p in plans for d in p[1]]
        if draws:
            if getattr(self, '_noise', None) is None or self._noise.dtype != first.dtype:
                self._noise = _NoiseStage(first.dtype)
            noise = self._noise.upload(draws)
            row0 = np.cumsum([0] + [len(p[0]) for p in plans])
            lib, dtc, stream = _lib.lib(), _lib.dtype_code(first.dtype), _lib.stream_handle()
            for k in range(max(len(p[0]) for p in plans)):
                todo = [(layer, p[0][k], noise[row0[i] + k]) for i, (layer, p) in enumerate(zip(layers, plans))
                        if len(p[0]) > k]
                steps = (_lib.Extrusion * len(todo))(*[layer._extrusion(w, x) for layer, w, x in todo])
                _lib.check(lib.hx_atmosphere_extrude_layers(steps, len(todo), dtc, stream),
                           'hx_atmosphere_extrude_layers')
                for layer, w, _ in todo:
                    layer._moved(w)
        n = len(layers)
        screens = [layer._shifted for layer in layers]
        if (self._combined is None or self._combined.dtype != first.dtype or
                self._combined.numel() != screens[0].numel()):
            self._combined = torch.empty_like(screens[0].reshape(-1))
        c = _lib.ctypes
        rings = (c.c_void_p * n)(*[_lib.dptr(layer._ring) for layer in layers])
        outs = (c.c_void_p * n)(*[_lib.dptr(x) for x in screens])
        r0, _ = _lib.iarr([layer._row0 for layer in layers])
        c0, _ = _lib.iarr([layer._col0 for layer in layers])
        taps_row = np.ascontiguousarray(np.concatenate([p[2] for p in plans]), np.float64)
        taps_col = np.ascontiguousarray(np.concatenate([p[3] for p in plans]), np.float64)
        P = c.POINTER(c.c_double)
        rc = _lib.lib().hx_atmosphere_shift_layers(rings, n, first.ny + 1, first.nx + 1, first.ny, first.nx,
                                                   c.cast(r0, c.POINTER(c.c_int)), c.cast(c0, c.POINTER(c.c_int)),
                                                   taps_row.ctypes.data_as(P), taps_col.ctypes.data_as(P), outs,
                                                   _lib.dptr(self._combined), _lib.dtype_code(first.dtype),
                                                   _lib.stream_handle())
        _lib.check(rc, 'hx_atmosphere_shift_layers')
        for layer in layers:
            layer._version += 1
        self._combined_key = tuple((id(layer), layer._version, s.data_ptr()) for layer, s in zip(layers, screens))

    def reset(self, make_independent_realization=False):
        for layer in self.layers:
            layer.reset(make_independent_realization)
        self._t = 0
        self.combined_screen()

    @property
    def t(self):
        return self._t

    @t.setter
    def t(self, t):
        self.evolve_until(t)

    def combined_screen(self):
        """The sum of the layers' current screens (radians at 1 m), a device tensor (npix,)."""
        screens = [layer._screen_tensor() for layer in self.layers]
        key = tuple((id(layer), getattr(layer, '_version', None), s.data_ptr())
                    for layer, s in zip(self.layers, screens))
        if self._combined is not None and key == self._combined_key and None not in (k[1] for k in key):
            return self._combined
        dt = screens[0].dtype
        if any(s.dtype != dt or s.numel() != screens[0].numel() for s in screens):
            raise ValueError('the layers must share their grid and screen dtype')
        if self._combined is None or self._combined.dtype != dt or self._combined.numel() != screens[0].numel():
            self._combined = torch.empty_like(screens[0].reshape(-1))
        start = 0
        while start < len(screens):
            # up to 8 screens a launch; past the first launch, 7 more plus the running sum
            part = screens[start:start + (8 if start == 0 else 7)]
            ptrs = (_lib.ctypes.c_void_p * (len(part) + (start > 0)))()
            for i, s in enumerate(part):
                ptrs[i] = _lib.dptr(s)
            if start > 0:
                ptrs[len(part)] = _lib.dptr(self._combined)
            start += len(part)
            rc = _lib.lib().hx_atmosphere_combine(ptrs, len(ptrs), screens[0].numel(), _lib.dptr(self._combined),
                                                  _lib.dtype_code(dt), _lib.stream_handle())
            _lib.check(rc, 'hx_atmosphere_combine')
        self._combined_key = key
        return self._combined

    def phase_for(self, wavelength):
        if self._scintillation:
            raise ValueError('Cannot get the unwrapped phase for an atmosphere with scintillation.')
        return Field(self.combined_screen() / wavelength, self.layers[0].input_grid)

    def _pure_phase_screen(self):
        """The summed screen when the forward is exp(i s / wavelength) (no scintillation), else None."""
        return None if self._scintillation else self.combined_screen()

    def _apply(self, wf, sign):
        e = as_tensor(wf.electric_field)
        s = self.combined_screen()
        if torch.is_grad_enabled() and e.requires_grad:
            from .autograd import phase_apply
            out = phase_apply(e, s, sign / wf.wavelength)
        else:
            out = apply_phase(e, s, sign / wf.wavelength)
        return wf._carry(Field(out, wf.electric_field.grid))

    def forward(self, wavefront):
        if self._scintillation:
            elements = self._elements or self.calculate_propagators()
            for el in elements:
                wavefront = el.forward(wavefront)
            return wavefront
        return self._apply(wavefront, 1.0)

    def backward(self, wavefront):
        if self._scintillation:
            elements = self._elements or self.calculate_propagators()
            for el in reversed(elements):
                wavefront = el.backward(wavefront)
            return wavefront
        return self._apply(wavefront, -1.0)
