"""Pyramid wavefront-sensor optics against the reference's own propagation (golden vectors from
hcipy/wavefront_sensing/pyramid.py): forward at two wavelengths (a dispersive pyramid), backward, complex64.
Tolerances: complex128 1e-10 relative; complex64 1e-5.
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
