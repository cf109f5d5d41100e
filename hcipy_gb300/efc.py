"""Electric-field conjugation on the device: the regularised inverses of hcipy/util/matrix_inversion.py, the
poke Jacobian of the reference's electric-field-conjugation tutorial measured with batches of DM commands, and
the EFC update.

The propagation of the pokes runs through this package's transforms (DM phase kernel, split or FP32 MFTs, the
Lyot chain), a batch of command vectors per call.  What remains here is small: the SVD of the (2 n_dz x n_act)
Jacobian in float64 (cuSOLVER through ``torch.linalg.svd``), the dark-zone gather and the control
matrix-vector product.  Matrices given as numpy arrays come back as numpy arrays; device tensors stay on the
device.
"""
import numpy as np
import torch

from . import _lib
from .field import Field, as_tensor as _to_device

_DEVICE = 'cuda'


def _device_matrix(m):
    """(device float64/complex128 tensor, was-a-tensor flag)."""
    if isinstance(m, Field):
        m = m.data
    if isinstance(m, torch.Tensor):
        dt = torch.complex128 if m.is_complex() else torch.float64
        return m.to(device=_DEVICE, dtype=dt), True
    a = np.asarray(m)
    a = a.astype(np.complex128 if np.iscomplexobj(a) else np.float64)
    return torch.from_numpy(a).to(_DEVICE), False


def _back(t, as_tensor):
    return t if as_tensor else t.cpu().numpy()


def _thin_svd(m):
    """M = U diag(S) Vt (S descending).  A tall matrix (a Jacobian: twice the dark-zone pixels by the actuators)
    goes through a QR factorisation first, M = Q R, so the SVD proper runs on the small square R and U = Q U_R;
    a wide one through its transpose.  On the device the square SVD uses cuSOLVER's QR-iteration driver."""
    rows, cols = m.shape[-2], m.shape[-1]
    kw = {'driver': 'gesvd'} if m.is_cuda else {}
    if rows >= 2 * cols:
        q, r = torch.linalg.qr(m, mode='reduced')
        ur, s, vt = torch.linalg.svd(r, full_matrices=False, **kw)
        return q @ ur, s, vt
    if cols >= 2 * rows:
        u, s, vt = _thin_svd(m.mT)
        return vt.mT, s, u.mT
    return torch.linalg.svd(m, full_matrices=False, **kw)


class SVD(object):
    """Thin singular value decomposition on the device (hcipy/util/singular_value_decomposition.py:7-120).

    ``svd`` is (U, S, Vt) with M = U diag(S) Vt and S descending.  With ``num_modes`` only that many of the
    largest singular modes are kept; the reference computes them with a sparse partial solver, here they are
    the leading part of the full decomposition.
    """

    def __init__(self, matrix=None, num_modes=None):
        if matrix is None:
            raise ValueError('You need to supply a matrix.')
        m, self._tensor = _device_matrix(matrix)
        u, s, vt = _thin_svd(m)
        if num_modes is not None:
            num_modes = int(num_modes)
            u, s, vt = u[:, :num_modes], s[:num_modes], vt[:num_modes]
        self._svd = (u, s, vt)
        self._num_modes = num_modes

    @property
    def svd(self):
        return tuple(_back(t, self._tensor) for t in self._svd)

    @property
    def num_modes(self):
        return self._num_modes if self._num_modes is not None else int(self._svd[1].numel())

    @property
    def U(self):  # noqa: N802
        return _back(self._svd[0], self._tensor)

    @property
    def S(self):  # noqa: N802
        return _back(self._svd[1], self._tensor)

    @property
    def singular_values(self):
        return self.S

    @property
    def Vt(self):  # noqa: N802
        return _back(self._svd[2], self._tensor)


def _factors(matrix, svd):
    """Device (U, S, Vt) of ``matrix`` (or of the given decomposition) and whether to return a tensor."""
    as_tensor = isinstance(matrix, (torch.Tensor, Field))
    if svd is None:
        svd = SVD(matrix)
    if isinstance(svd, SVD):
        u, s, vt = svd._svd
    else:
        u, s, vt = (_device_matrix(t)[0] for t in svd.svd)
    return u, s, vt, as_tensor


def inverse_tikhonov(M, rcond=1e-15, svd=None):
    """Tikhonov-regularised inverse (matrix_inversion.py:68-98): Vt^T diag(s / (s^2 + (rcond s_max)^2)) U^T.

    The same matrix is (M^T M + a^2 I)^-1 M^T with a = rcond s_max.  For a real M, no decomposition given and
    rcond >= 1e-4 it is computed that way: the Gram matrix, its largest eigenvalue and a Cholesky solve, all
    BLAS3-shaped, where the SVD takes ten times longer on the device.  The regularised Gram matrix has condition
    number at most 1 + rcond^-2, so the float64 result keeps at least 8 significant digits; a smaller rcond,
    complex matrices or a given ``svd`` go through the SVD as in the reference.
    """
    if svd is None and float(rcond) >= 1e-4:
        m, as_tensor = _device_matrix(M)
        if not m.is_complex():
            g = m.mT @ m
            a2 = float(rcond)**2 * float(torch.linalg.eigvalsh(g)[-1])
            g.diagonal().add_(a2)
            return _back(torch.cholesky_solve(m.mT.contiguous(), torch.linalg.cholesky(g)), as_tensor)
    u, s, vt, as_tensor = _factors(M, svd)
    s_inv = s / (s**2 + (float(rcond) * s.max())**2)
    return _back((vt.T * s_inv.to(vt.dtype)) @ u.T, as_tensor)


def inverse_truncated(M, rcond=1e-15, svd=None):
    """Inverse without the modes whose singular value is at most rcond s_max (matrix_inversion.py:38-66)."""
    u, s, vt, as_tensor = _factors(M, svd)
    keep = s.abs() > float(rcond) * s.max()
    s_inv = torch.where(keep, 1.0 / torch.where(keep, s, torch.ones_like(s)), torch.zeros_like(s))
    return _back((vt.T * s_inv.to(vt.dtype)) @ u.T, as_tensor)


def inverse_truncated_modal(M, num_modes, svd=None):
    """Inverse on the num_modes largest singular modes (matrix_inversion.py:3-36)."""
    num_modes = int(num_modes)
    if svd is None:
        svd = SVD(M, num_modes)
    u, s, vt, as_tensor = _factors(M, svd)
    u, s, vt = u[:, :num_modes], s[:num_modes], vt[:num_modes]
    return _back((vt.T / s.to(vt.dtype)) @ u.T, as_tensor)


def _mask(dark_zone):
    dz = dark_zone.data if isinstance(dark_zone, Field) else dark_zone
    return torch.as_tensor(np.asarray(dz) if not isinstance(dz, torch.Tensor) else dz).reshape(-1)


def _dark_zone_index(dz):
    """Indices of the dark-zone pixels, on the device."""
    return torch.nonzero(dz.to(_DEVICE).bool()).reshape(-1)


def _check_pixels(n, npix):
    """Host-side size check before any device gather."""
    if n != npix:
        raise ValueError('The field has %d pixels per vector but the dark-zone mask has %d.' % (n, npix))


def poke_jacobian(measure, dark_zone, num_modes, epsilon, num_amplitudes=2, batch=32, dtype=torch.float64):
    """The EFC tutorial's poke Jacobian, measured on the device in batches of command vectors.

    ``measure(commands)`` takes a (B, num_modes) tensor of DM commands and returns the (B, npix) focal-plane
    fields (e.g. DM -> coronagraph -> lens).  Per mode i the response is sum_a a E(a e_i) / var(amps) with
    amps = linspace(-epsilon, epsilon, num_amplitudes), restricted to the dark zone; the result stacks the real
    parts over the imaginary parts: a (2 n_dz, num_modes) float64 device tensor.  With two amplitudes it is
    (E(+eps) - E(-eps)) / eps, the convention the reference's loop gain is tuned for.  ``batch`` modes
    (batch x num_amplitudes command vectors) go through the chain per call.
    """
    dz = _mask(dark_zone)
    npix, n_dz = int(dz.numel()), int(dz.bool().sum())
    epsilon, num_modes, num_amplitudes = float(epsilon), int(num_modes), int(num_amplitudes)
    amps = torch.linspace(-epsilon, epsilon, num_amplitudes, dtype=torch.float64)
    var = float(amps.var(unbiased=False))
    idx = jac = None
    amps_dev = amps.to(_DEVICE)
    for start in range(0, num_modes, batch):
        nb = min(batch, num_modes - start)
        # the pokes are written on the device (a host-built batch would be a synchronous copy per batch)
        cmds = torch.zeros((nb, num_amplitudes, num_modes), dtype=torch.float64, device=_DEVICE)
        rows = torch.arange(nb, device=_DEVICE)
        cmds[rows, :, start + rows] = amps_dev
        fields = measure(cmds.reshape(nb * num_amplitudes, num_modes).to(dtype=dtype))
        fields = torch.as_tensor(fields.data if isinstance(fields, Field) else fields)
        if fields.numel() != nb * num_amplitudes * npix:
            raise ValueError('measure() returned %s for %d command vectors of a %d-pixel focal grid.'
                             % (tuple(fields.shape), nb * num_amplitudes, npix))
        if jac is None:
            idx = _dark_zone_index(dz)
            jac = torch.empty((2 * n_dz, num_modes), dtype=torch.float64, device=_DEVICE)
        f = fields.reshape(nb, num_amplitudes, npix).index_select(2, idx).to(torch.complex128)
        resp = (amps_dev.view(1, -1, 1) * f).sum(1) / var
        jac[:n_dz, start:start + nb] = resp.real.T
        jac[n_dz:, start:start + nb] = resp.imag.T
    return jac


def efc_step(efc_matrix, field, dark_zone, actuators, gain):
    """One EFC update (the tutorial's loop body): x = [Re E_dz, Im E_dz], actuators - gain * (efc_matrix . x).

    One launch of ``hx_efc_step`` (the dark-zone gather, the matrix product and the update, float-float
    arithmetic); the EFC matrix (from ``inverse_tikhonov`` and friends, computed once per Jacobian) stays on the
    device in float64."""
    dz = _mask(dark_zone)
    e = field.data if isinstance(field, Field) else field
    e = torch.as_tensor(e).reshape(-1)
    _check_pixels(e.numel(), int(dz.numel()))
    idx = _dark_zone_index(dz).to(torch.int32).contiguous()
    m, _ = _device_matrix(efc_matrix)
    return _efc_update(m.to(torch.float64).contiguous(), e, idx, actuators, gain)


def _efc_update(m, e, idx, actuators, gain):
    """hx_efc_step with the float64 matrix and the int32 dark-zone indices already on the device."""
    e = _to_device(e)
    if e.dtype not in (torch.complex64, torch.complex128):
        e = e.to(torch.complex128)
    e = e.contiguous()
    if m.shape[1] != 2 * idx.numel():
        raise ValueError('The EFC matrix has %d columns; the dark zone needs %d.' % (m.shape[1], 2 * idx.numel()))
    a = torch.as_tensor(actuators.data if isinstance(actuators, Field) else actuators)
    a = a.to(device=_DEVICE, dtype=torch.float64).contiguous()
    if a.numel() != m.shape[0]:
        raise ValueError('%d actuators for an EFC matrix of %d rows.' % (a.numel(), m.shape[0]))
    out = torch.empty_like(a)
    rc = _lib.lib().hx_efc_step(_lib.dptr(m), int(m.shape[0]), int(idx.numel()), _lib.dptr(e), _lib.dtype_code(e.dtype),
                                _lib.dptr(idx), _lib.dptr(a), float(gain), _lib.dptr(out), _lib.stream_handle())
    _lib.check(rc, 'hx_efc_step')
    return out


def run_efc(measure, dark_zone, efc_matrix, actuators, iterations, gain=0.5):
    """The tutorial's EFC loop on the device: ``iterations`` times measure the field at the current commands
    (``measure`` takes one (num_modes,) command tensor and returns the focal-plane field) and update them.
    Returns the list of commands applied and the list of fields measured."""
    a = torch.as_tensor(actuators).to(device=_DEVICE, dtype=torch.float64)
    dz = _mask(dark_zone)
    idx = _dark_zone_index(dz).to(torch.int32).contiguous()  # once: the loop then never waits on the device
    m = _device_matrix(efc_matrix)[0].to(torch.float64).contiguous()
    history, fields = [], []
    for _ in range(iterations):
        e = measure(a)
        history.append(a.clone())
        fields.append(e)
        f = e.data if isinstance(e, Field) else e
        f = torch.as_tensor(f).reshape(-1)
        _check_pixels(f.numel(), int(dz.numel()))
        a = _efc_update(m, f, idx, a, gain)
    return history, fields
