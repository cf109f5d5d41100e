"""Electric-field conjugation on the device against the reference run on a seeded 32^2 case (tests/golden/efc.npz):
the poke Jacobian measured through the DM, the Lyot coronagraph and the lens in batches of commands, the
Tikhonov control matrix (float64 SVD on the device) and five EFC iterations.

Tolerances: the Jacobian is a difference quotient over pokes of 1e-3 wavelengths, so a field error e shows up
as ~e/1e-3 in it.  Split precision with complex128 fields (errors ~1e-12 of the peak): 1e-6 relative; FP32 with
complex64 fields (~1e-7 of the peak): 1e-2.  The float64 inverses agree to 1e-9.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def _grid(g, p):
    return hg.CartesianGrid(hg.RegularCoords(g[p + '_delta'], g[p + '_dims'], g[p + '_zero']))


def _chain(g, precision):
    pupil, fpm_grid, focal = _grid(g, 'pupil'), _grid(g, 'fpm'), _grid(g, 'focal')
    lyot = hg.LyotCoronagraph(pupil, hg.Field(g['fpm'], fpm_grid), hg.Field(g['stop'], pupil), precision=precision)
    prop = hg.FraunhoferPropagator(pupil, focal, precision=precision)
    split = precision == 'split'
    dm = hg.DeformableMirror(hg.ModeBasis(g['influence'], pupil), dtype=torch.float64 if split else torch.float32)
    cdt = np.complex128 if split else np.complex64

    def measure(e0):
        e0 = torch.from_numpy(np.asarray(e0, cdt)).cuda()

        def f(cmds):
            dm.actuators = cmds
            return prop.forward(lyot.forward(dm.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0)))).electric_field.data
        return f
    return measure


def test_inverses_match_reference():
    g = load_golden('efc')
    m = g['M']
    assert rel_err(hg.inverse_tikhonov(m, 1e-3), g['M_tikhonov']) < 1e-9
    assert rel_err(hg.inverse_truncated(m, 1e-4), g['M_truncated']) < 1e-9
    assert rel_err(hg.inverse_truncated_modal(m, 5), g['M_modal']) < 1e-9
    # device tensors stay on the device; a precomputed SVD is reused
    mt = torch.from_numpy(m).cuda()
    svd = hg.SVD(mt)
    out = hg.inverse_tikhonov(mt, 1e-3, svd=svd)
    assert out.is_cuda and rel_err(out.cpu().numpy(), g['M_tikhonov']) < 1e-9
    assert rel_err(hg.inverse_tikhonov(g['jacobian'], g['rcond']), g['efc_matrix']) < 1e-9


@pytest.mark.parametrize('precision,tol', [('split', 1e-6), ('fp32', 1e-2)])
def test_poke_jacobian_matches_reference(precision, tol):
    g = load_golden('efc')
    measure = _chain(g, precision)(g['aperture'])
    nact = g['influence'].shape[1]
    dtype = torch.float64 if precision == 'split' else torch.float32
    jac = hg.poke_jacobian(measure, g['dark_zone'], nact, float(g['epsilon']), batch=7, dtype=dtype)
    assert jac.shape == g['jacobian'].shape
    assert rel_err(jac.cpu().numpy(), g['jacobian']) < tol, rel_err(jac.cpu().numpy(), g['jacobian'])


def test_efc_loop_matches_reference():
    g = load_golden('efc')
    measure = _chain(g, 'split')(g['aberration'])
    em = hg.inverse_tikhonov(torch.from_numpy(g['jacobian']).cuda(), float(g['rcond']))
    hist, fields = hg.run_efc(lambda a: measure(a[None])[0], g['dark_zone'], em, g['actuators'][0],
                              len(g['actuators']), float(g['gain']))
    for a, ref in zip(hist, g['actuators']):
        assert rel_err(a.cpu().numpy(), ref) < 1e-6 if np.any(ref) else not torch.any(a)
    dz = torch.from_numpy(g['dark_zone']).cuda()
    ni = [float((f[dz].abs()**2).mean()) / float(g['peak']) for f in fields]
    assert np.allclose(ni, g['dark_zone_ni'], rtol=1e-6)
    assert ni[-1] < 0.5 * ni[0]


@pytest.mark.parametrize('dtype', [np.complex128, np.complex64])
@pytest.mark.parametrize('nact,npix,n_dz', [(952, 65536, 6702), (37, 400, 1), (5, 64, 0)])
def test_efc_step_kernel_matches_float64(dtype, nact, npix, n_dz):
    """hx_efc_step (one launch: dark-zone gather, float-float matrix product, update) against the numpy float64
    form a - gain (M [Re E_dz, Im E_dz]), at the size of the 952-actuator, 6702-pixel dark zone and at ragged and
    empty dark zones.  Bound: 1e-12 of |a| + gain |M| |x| per actuator (float-float keeps ~46 bits)."""
    rng = np.random.default_rng(nact + n_dz)
    dz = np.zeros(npix, bool)
    dz[rng.choice(npix, n_dz, replace=False)] = True
    m = rng.standard_normal((nact, 2 * n_dz))
    e = (rng.standard_normal(npix) + 1j * rng.standard_normal(npix)).astype(dtype)
    a = rng.standard_normal(nact)
    gain = 0.37
    x = np.concatenate((e[dz].real, e[dz].imag)).astype(np.float64)
    ref = a - gain * (m @ x)
    bound = np.abs(a) + gain * (np.abs(m) @ np.abs(x))
    got = hg.efc_step(torch.from_numpy(m).cuda(), torch.from_numpy(e).cuda(), dz, torch.from_numpy(a).cuda(), gain)
    assert got.is_cuda and got.dtype == torch.float64
    err = np.abs(got.cpu().numpy() - ref) / bound
    assert err.max() < 1e-12, err.max()
    # the host-array form returns the same
    again = hg.efc_step(m, e, dz, a, gain)
    assert torch.equal(again.cpu(), got.cpu())
