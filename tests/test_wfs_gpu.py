"""Pyramid wavefront-sensor optics against the reference's own propagation (golden vectors from
hcipy/wavefront_sensing/pyramid.py): forward at two wavelengths (a dispersive pyramid), backward, complex64; the
modulated sensor (both methods) and the tip-tilt mirror.
Tolerances: complex128 1e-10 relative; complex64 1e-5 (2e-5 for the modulated sensor, whose phases reach ~110 rad
before they are reduced).
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def test_pyramid_matches_reference():
    g = load_golden('pyramid')
    pupil = hg.make_pupil_grid(48, 1.0)
    wfs_grid = hg.make_pupil_grid(96, 2.0)
    pwfs = hg.PyramidWavefrontSensorOptics(pupil, wfs_grid, separation=1.0, pupil_diameter=1.0, wavelength_0=1.0,
                                           refractive_index=lambda wl: 1.5 + 0.01 * (wl - 1.0))
    assert np.array_equal(np.asarray(pwfs.focal_grid.dims), g['focal_dims'])
    assert np.allclose(pwfs.focal_grid.delta, g['focal_delta'], rtol=0, atol=1e-15)
    for k in range(2):
        wl = float(g['wavelength_%d' % k])
        out = pwfs.forward(hg.Wavefront(hg.Field(g['E'], pupil), wl)).electric_field.numpy()
        assert rel_err(out, g['fwd_%d' % k]) < 1e-10, k
    back = pwfs.backward(hg.Wavefront(hg.Field(g['G'], wfs_grid), 1.0)).electric_field.numpy()
    assert rel_err(back, g['bwd']) < 1e-10
    out32 = pwfs.forward(hg.Wavefront(hg.Field(g['E'].astype(np.complex64), pupil), 1.0)).electric_field.numpy()
    assert out32.dtype == np.complex64 and rel_err(out32, g['fwd_0']) < 1e-5
    with pytest.raises(ValueError):
        hg.PyramidWavefrontSensorOptics(pupil, wfs_grid, q=1)


def test_surface_apodizer_dispersion():
    """SurfaceApodizer (apodization.py:64-102): exp(+-i (n(lambda) - 1) sag 2 pi / lambda)."""
    grid = hg.make_pupil_grid(16, 1.0)
    rng = np.random.default_rng(1)
    sag = rng.standard_normal(grid.size) * 1e-7
    e = rng.standard_normal(grid.size) + 1j * rng.standard_normal(grid.size)
    ap = hg.SurfaceApodizer(sag, lambda wl: 1.45 + 1e-2 / wl)
    for wl in (0.5, 0.8):
        out = ap.forward(hg.Wavefront(hg.Field(e, grid), wl)).electric_field.numpy()
        ref = e * np.exp(1j * (1.45 + 1e-2 / wl - 1) * sag * 2 * np.pi / wl)
        assert rel_err(out, ref) < 1e-13
        back = ap.backward(hg.Wavefront(hg.Field(out, grid), wl)).electric_field.numpy()
        assert rel_err(back, e) < 1e-13


def _modulated(g, fast):
    pupil = hg.make_pupil_grid(32, 1.0)
    pwfs = hg.PyramidWavefrontSensorOptics(pupil, hg.make_pupil_grid(40, 2.0), separation=1.0, pupil_diameter=1.0,
                                           wavelength_0=1.0, refractive_index=lambda wl: 1.5 + 0.01 * (wl - 1.0))
    return pupil, hg.ModulatedPyramidWavefrontSensorOptics(pwfs, float(g['modulation']), num_steps=int(g['num_steps']),
                                                           fast_modulation_method=fast)


def _steps(wfs):
    return np.stack([w.electric_field.numpy() for w in wfs])


@pytest.mark.parametrize('fast', [False, True])
def test_modulated_pyramid_matches_reference(fast):
    """ModulatedPyramidWavefrontSensorOptics (pyramid.py:10-91): every modulation step against the reference, in
    complex128 and complex64; a wavefront holding two fields gives each field's steps."""
    g = load_golden('modulated_pyramid')
    pupil, mod = _modulated(g, fast)
    steps = int(g['num_steps'])
    cases = [(float(g['wavelength_%d' % k]), g['fast_%d' % k]) for k in range(2)] if fast else [(1.0, g['slow'])]
    for wl, ref in cases:
        out = mod.forward(hg.Wavefront(hg.Field(g['E'], pupil), wl))
        assert len(out) == steps and out[0].wavelength == wl
        assert rel_err(_steps(out), ref) < 1e-10, wl
    wl, ref = cases[0]
    out32 = _steps(mod.forward(hg.Wavefront(hg.Field(g['E'].astype(np.complex64), pupil), wl)))
    assert out32.dtype == np.complex64 and rel_err(out32, ref) < 2e-5
    e2 = torch.from_numpy(np.stack([g['E'], g['E'] * np.exp(0.3j)])).cuda()
    both = mod.forward(hg.Wavefront(hg.Field(e2, pupil), wl))
    assert tuple(both[0].electric_field.data.shape) == (2, 1600)
    for j in range(2):
        one = mod.forward(hg.Wavefront(hg.Field(e2[j].contiguous(), pupil), wl))
        for a, b in zip(both, one):
            assert torch.equal(a.electric_field.data[j], b.electric_field.data)
    if not fast:
        assert np.array_equal(mod.tip_tilt_mirror.actuators, g['positions'][-1])
    with pytest.raises(RuntimeError):
        mod.backward(out[0])


def test_tip_tilt_mirror_matches_reference():
    """TipTiltMirror (hcipy/optics/tip_tilt_mirror.py): one command against the reference, its backward undoing
    it, and a batch of commands in one call equal to the commands one by one."""
    g = load_golden('modulated_pyramid')
    pupil = hg.make_pupil_grid(32, 1.0)
    ttm = hg.TipTiltMirror(pupil)
    ttm.actuators = g['tip_tilt_command']
    out = ttm.forward(hg.Wavefront(hg.Field(g['E'], pupil), 0.8))
    assert rel_err(out.electric_field.numpy(), g['tip_tilt']) < 1e-12
    assert rel_err(ttm.backward(out).electric_field.numpy(), g['E']) < 1e-12
    cmds = torch.tensor([[1e-3, 0.0], [0.0, -2e-3], [3e-3, 1e-3]], dtype=torch.float64)
    ttm.actuators = cmds
    batch = ttm.forward(hg.Wavefront(hg.Field(g['E'], pupil), 0.8)).electric_field.data
    for k in range(3):
        ttm.actuators = cmds[k].numpy()
        one = ttm.forward(hg.Wavefront(hg.Field(g['E'], pupil), 0.8)).electric_field.data
        assert torch.equal(batch[k], one)
