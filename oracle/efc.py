"""Electric-field-conjugation arithmetic of the reference, restated in float64 numpy (test infrastructure only).

Regularised inverses follow hcipy/util/matrix_inversion.py; the poke Jacobian and the control step follow the
electric-field-conjugation tutorial (doc/tutorial_notebooks/ElectricFieldConjugation, the Jacobian and EFC-loop
cells).  Pinned against tests/golden/efc.npz, made by running the reference.
"""
import numpy as np


def _svd(m):
    return np.linalg.svd(np.asarray(m), full_matrices=False)


def inverse_tikhonov(m, rcond=1e-15):
    """matrix_inversion.py:68-98: V diag(s / (s^2 + (rcond s_max)^2)) U^T."""
    u, s, vt = _svd(m)
    s_inv = s / (s**2 + (rcond * s.max())**2)
    return (vt.T * s_inv) @ u.T


def inverse_truncated(m, rcond=1e-15):
    """matrix_inversion.py:38-66: modes with s <= rcond s_max are dropped."""
    u, s, vt = _svd(m)
    s_inv = np.where(np.abs(s) > rcond * s.max(), 1.0 / np.where(s == 0, 1.0, s), 0.0)
    return (vt.T * s_inv) @ u.T


def inverse_truncated_modal(m, num_modes):
    """matrix_inversion.py:3-36: the num_modes largest singular modes."""
    u, s, vt = _svd(m)
    return (vt[:num_modes].T / s[:num_modes]) @ u[:, :num_modes].T


def poke_jacobian(get_field, dark_zone, num_modes, epsilon, num_amplitudes=2):
    """The tutorial's Jacobian: per mode i, sum_a a E(a e_i) / var(amps) with amps = linspace(-eps, eps, n),
    restricted to the dark zone, real parts stacked over imaginary parts -> (2 n_dz, num_modes).

    With two amplitudes this is (E(+eps) - E(-eps)) / eps, twice the derivative; the reference's EFC gain is
    tuned with that convention.
    """
    amps = np.linspace(-epsilon, epsilon, num_amplitudes)
    cols = []
    for i in range(num_modes):
        resp = 0
        for a in amps:
            cmd = np.zeros(num_modes)
            cmd[i] = a
            resp = resp + a * np.asarray(get_field(cmd))
        resp = resp / np.var(amps)
        resp = resp[dark_zone]
        cols.append(np.concatenate((resp.real, resp.imag)))
    return np.array(cols).T


def efc_step(efc_matrix, field, dark_zone, actuators, gain):
    """The tutorial's EFC update: x = [Re E_dz, Im E_dz], actuators - gain * (efc_matrix . x)."""
    e = np.asarray(field)[dark_zone]
    x = np.concatenate((e.real, e.imag))
    return actuators - gain * (efc_matrix @ x)
