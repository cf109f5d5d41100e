"""Host-side logic that runs without a GPU: grids, FFT-grid algebra, the instance cache."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import grids as ogrids

import hcipy_gb300 as hg


def test_pupil_and_focal_grids_match_reference():
    g = load_golden('fraunhofer_cfg1')
    pupil = hg.make_pupil_grid(256, 1)
    focal = hg.make_focal_grid(q=4, num_airy=16)
    np.testing.assert_array_equal(pupil.dims, g['pupil_dims'])
    np.testing.assert_allclose(pupil.delta, g['pupil_delta'], rtol=0)
    np.testing.assert_allclose(pupil.zero, g['pupil_zero'], rtol=1e-15)
    np.testing.assert_array_equal(focal.dims, g['focal_dims'])
    np.testing.assert_allclose(focal.zero, g['focal_zero'], rtol=1e-15)
    assert pupil.weights == pytest.approx(g['pupil_weights'][0], rel=1e-15)
    assert pupil.shape == (256, 256)


@pytest.mark.parametrize('case', ['fft_0', 'fft_1', 'fft_2', 'fft_3'])
def test_fft_grid_algebra(case):
    g = load_golden(case)
    pupil = hg.make_pupil_grid(tuple(g['ingrid_dims']), tuple(g['ingrid_dims'] * g['ingrid_delta']))
    out = hg.make_fft_grid(pupil, float(g['q']), float(g['fov']), tuple(g['shift']))
    np.testing.assert_array_equal(out.dims, g['outgrid_dims'])
    np.testing.assert_allclose(out.delta, g['outgrid_delta'], rtol=1e-14)
    np.testing.assert_allclose(out.zero, g['outgrid_zero'], rtol=1e-12, atol=1e-14)
    q, fov, shift = hg.get_fft_parameters(out, pupil)
    again = hg.make_fft_grid(pupil, q, fov, shift)
    np.testing.assert_array_equal(again.dims, out.dims)
    np.testing.assert_allclose(again.zero, out.zero, rtol=1e-12, atol=1e-14)


def test_non_fft_grid_detected():
    pupil = hg.make_pupil_grid(64, 1)
    focal = hg.make_focal_grid(3.3, 8).scaled(2 * np.pi)
    assert not hg.is_fft_grid(focal, pupil)
    assert hg.is_fft_grid(hg.make_fft_grid(pupil, 2, 0.5), pupil)


def test_mft_supported_grids():
    pupil = hg.make_pupil_grid(16, 1)
    assert hg.MatrixFourierTransform.is_supported(pupil, hg.make_focal_grid(2, 4))
    un = hg.CartesianGrid(hg.UnstructuredCoords([np.zeros(3), np.ones(3)]))
    assert not hg.MatrixFourierTransform.is_supported(un, pupil)
    with pytest.raises(ValueError):
        hg.MatrixFourierTransform.check_if_supported(pupil, hg.make_uniform_grid(5, 1))


def test_separated_weights_match_reference_formula():
    g = hg.CartesianGrid(hg.SeparatedCoords([np.array([0.0, 0.1, 0.3, 0.6]), np.array([1.0, 1.5, 2.5])]))
    w = g.weights
    wx = np.array([0.1, 0.15, 0.25, 0.3])
    wy = np.array([0.5, 0.75, 1.0])
    np.testing.assert_allclose(w, (wy[:, None] * wx[None, :]).ravel())


def test_agnostic_cache_fifo():
    made = []

    class Probe(hg.AgnosticOpticalElement):
        def make_instance(self, inst, ig, og, wl):
            made.append(wl)

        def get_output_grid(self, ig, wl):
            return ig

    p = Probe(max_in_cache=3)
    g = hg.make_pupil_grid(8)
    for wl in [1.0, 1.1, 1.2, 1.0, 1.3, 1.0]:
        p.get_instance_data(g, None, wl)
    # 1.0 hit once, evicted by 1.3 (FIFO of 3), then rebuilt.
    assert made == [1.0, 1.1, 1.2, 1.3, 1.0]
    assert len(p._instances) == 3


def test_oracle_grid_factories_agree_with_package():
    a = hg.make_focal_grid(2.5, (5, 7))
    b = ogrids.make_focal_grid(2.5, (5, 7))
    np.testing.assert_array_equal(a.dims, b.dims)
    np.testing.assert_allclose(a.zero, b.zero)


def test_efc_rejects_mismatched_fields(monkeypatch):
    """The EFC helpers check the field size against the dark-zone mask on the host, before any device gather
    (host tensors stand in for the device here)."""
    import torch
    from hcipy_gb300 import efc
    monkeypatch.setattr(efc, '_DEVICE', 'cpu')
    dz = np.zeros(16, bool)
    dz[3] = True
    with pytest.raises(ValueError):
        efc.efc_step(np.zeros((2, 2)), torch.zeros(1, dtype=torch.complex128), dz, np.zeros(2), 0.5)
    with pytest.raises(ValueError):
        efc.poke_jacobian(lambda c: torch.zeros(c.shape[0], 4, dtype=torch.complex128), torch.from_numpy(dz), 2,
                          1e-3)


# rcond = 1e-15 is the plain pseudo-inverse of a matrix of condition ~1e8: two SVD algorithms (QR first, or not)
# agree there only to ~condition x machine epsilon.
@pytest.mark.parametrize('rcond,tol', [(1e-2, 1e-11), (1e-3, 1e-9), (1e-5, 1e-9), (1e-15, 1e-7)])
def test_tikhonov_paths_agree_with_the_svd_form(monkeypatch, rcond, tol):
    """inverse_tikhonov's Gram/Cholesky form (rcond >= 1e-4) and its SVD form (smaller rcond) against the numpy
    restatement of the reference's SVD formula, on an ill-conditioned matrix (host tensors stand in for the
    device)."""
    import torch
    from conftest import rel_err
    from hcipy_gb300 import efc
    from oracle import efc as oefc
    monkeypatch.setattr(efc, '_DEVICE', 'cpu')
    rng = np.random.default_rng(5)
    m = rng.standard_normal((60, 16)) @ np.diag(np.logspace(0, -8, 16)) @ rng.standard_normal((16, 16))
    assert rel_err(efc.inverse_tikhonov(m, rcond), oefc.inverse_tikhonov(m, rcond)) < tol
    out = efc.inverse_tikhonov(torch.from_numpy(m), rcond)
    assert isinstance(out, torch.Tensor) and rel_err(out.numpy(), oefc.inverse_tikhonov(m, rcond)) < tol


def test_jones_stokes_matches_the_mueller_form():
    """The polarised wavefront's Stokes parameters (``optics.jones_stokes``, torch on any device) against the
    oracle's Mueller matrix A (J kron J*) A^-1 applied to the input Stokes vector (wavefront.py:103-235), on the
    CPU; any subset of rows equals the full computation."""
    import torch
    from hcipy_gb300.optics import jones_stokes
    from oracle import optics as ooptics
    rng = np.random.default_rng(4)
    j = rng.standard_normal((2, 2, 50)) + 1j * rng.standard_normal((2, 2, 50))
    s = np.array([1.0, 0.3, -0.2, 0.1])
    got = torch.stack(jones_stokes(torch.from_numpy(j), s)).numpy()
    ref = ooptics.stokes_parameters(j, s)
    assert np.max(np.abs(got - ref)) < 1e-14 * np.max(np.abs(ref))
    for k in range(4):
        assert np.array_equal(jones_stokes(torch.from_numpy(j), s, (k,))[0].numpy(), got[k])


def test_vector_vortex_coronagraph_sets_are_shared_and_bounded(monkeypatch):
    """The vector vortex builds its three scalar coronagraphs once per (grid, retardance): wavelengths with the
    same retardance share them, and at most as many sets as the instance cache holds are kept (first in, first
    out).  Host logic only: the scalar coronagraph is replaced by a recorder."""
    from hcipy_gb300 import coronagraphy
    built = []

    class Recorder(object):
        def __init__(self, grid, mask, *args):
            built.append(mask)

    monkeypatch.setattr(coronagraphy, 'MultiScaleCoronagraph', Recorder)
    grid = hg.make_pupil_grid(8, 1.0)
    fixed = hg.VectorVortexCoronagraph(2)
    a = fixed.get_instance_data(grid, None, 1.0)
    b = fixed.get_instance_data(grid, None, 1.3)
    assert a is not b and a.entries is b.entries and len(built) == 3
    chromatic = hg.VectorVortexCoronagraph(2, phase_retardation=lambda wl: np.pi * wl)
    for k in range(14):
        chromatic.get_instance_data(grid, None, 1.0 + 0.01 * k)
    assert len(chromatic._entries) == chromatic._max_in_cache == 11
    assert len(built) == 3 + 3 * 14


def test_planner_picks_the_reference_method():
    """make_fourier_transform(planner='estimate') ranks the methods with the reference's operation counts and time
    model: over 264 grid pairs (pupils of 16^2-2048^2 and rectangular ones; FFT output grids with q 1-16 and fov
    1-0.1; focal grids that are not FFT grids) every supported method's expected time equals the reference's
    (fourier_transform.py:217-300) and the pick is the reference's (it never picks its naive DFT here)."""
    from hcipy_gb300.fourier import _planned_methods
    g = load_golden('planner')
    methods = [str(m) for m in g['methods']]
    for i in range(len(g['best'])):
        pupil = hg.make_pupil_grid(tuple(int(d) for d in g['dims'][i]), tuple(float(d) for d in g['diameter'][i]))
        _, q, x, focal = g['params'][i]
        if focal:
            out = hg.make_focal_grid(q, x, spatial_resolution=1.0).scaled(
                2 * np.pi / np.max(np.asarray(pupil.delta) * np.asarray(pupil.dims)))
            _, expected, _, _ = _planned_methods(pupil, out, 1, 1, 0, 'estimate')
        else:
            _, expected, _, _ = _planned_methods(pupil, None, q, x, 0, 'estimate')
        for k, m in enumerate(methods):
            ref = g['times'][i, k]
            if m == 'naive':
                continue
            if np.isnan(ref):
                assert m not in expected, (i, m)
            else:
                assert abs(expected[m] - ref) <= 1e-12 * ref, (i, m, expected[m], ref)
        assert min(expected, key=expected.get) == methods[int(g['best'][i])], i


def test_fft_grid_algebra_sweep():
    """make_fft_grid and get_fft_parameters (fast_fourier_transform.py:23-154) against the reference over 270
    cases: square, rectangular and odd pupils, q 1-8 (including 1.5), fov 1-0.3, scalar and per-axis shifts."""
    g = load_golden('fft_grids')
    for r in g['rows']:
        dims, diam = tuple(int(d) for d in r[0:2]), tuple(r[2:4])
        q, fov, shift = r[4], r[5], tuple(r[6:8])
        pupil = hg.make_pupil_grid(dims, diam)
        out = hg.make_fft_grid(pupil, q, fov, shift)
        np.testing.assert_array_equal(out.dims, r[10:12])
        np.testing.assert_allclose(out.delta, r[8:10], rtol=1e-15)
        np.testing.assert_allclose(out.zero, r[12:14], rtol=1e-13, atol=1e-13)
        qq, ff, ss = hg.get_fft_parameters(out, pupil)
        np.testing.assert_allclose(np.broadcast_to(qq, (2,)), r[14:16], rtol=1e-12)
        np.testing.assert_allclose(np.broadcast_to(ff, (2,)), r[16:18], rtol=1e-12)
        np.testing.assert_allclose(np.broadcast_to(ss, (2,)), r[18:20], rtol=1e-12, atol=1e-12)


def test_grid_factories_and_turbulence_helpers_match_reference():
    """make_uniform_grid / make_pupil_grid / make_focal_grid / make_focal_grid_from_pupil_grid over odd and even
    sizes, centres, has_center and every way of giving the focal sampling (hcipy/field/util.py:68-318); the Cn^2 <-> Fried-parameter conversions, the
    von Karman PSD and phase covariance (hcipy/atmosphere/atmospheric_model.py:321-399)."""
    from hcipy_gb300.atmosphere import von_karman_covariance
    g = load_golden('host_functions')
    grids = []
    for dims, extent, center, has_center in [(8, 1.0, 0, False), (9, 1.0, 0, False), (9, 2.0, 0, True),
                                             (10, 2.0, 0, True), ((6, 7), (1.0, 1.4), (0.1, -0.3), False),
                                             ((6, 7), (1.0, 1.4), (0.1, -0.3), True)]:
        grids.append(hg.make_uniform_grid(dims, extent, center, has_center))
    for dims, diam in [(64, 1.0), (65, 2.0), ((40, 30), (1.0, 0.75))]:
        grids.append(hg.make_pupil_grid(dims, diam))
    for kw in [dict(q=4, num_airy=16), dict(q=3.3, num_airy=(8, 5.5)), dict(q=2, num_airy=10, spatial_resolution=0.5),
               dict(q=4, num_airy=8, pupil_diameter=8.0, focal_length=20.0, reference_wavelength=1.6e-6),
               dict(q=5, num_airy=6, f_number=12.0, reference_wavelength=7e-7)]:
        grids.append(hg.make_focal_grid(**kw))
    for dims, diam, kw in [(64, 1.0, dict(q=4, num_airy=16)),
                           ((40, 30), (1.0, 0.75), dict(q=3, num_airy=(8, 6), focal_length=2.0, wavelength=0.5)),
                           (33, 2.0, dict(q=2))]:
        grids.append(hg.make_focal_grid_from_pupil_grid(hg.make_pupil_grid(dims, diam), **kw))
    assert len(grids) == len(g['grids'])
    for grid, ref in zip(grids, g['grids']):
        n = int(ref[0])
        assert grid.ndim == n
        np.testing.assert_allclose(grid.delta, ref[1:1 + n], rtol=1e-15)
        np.testing.assert_array_equal(grid.dims, ref[3:3 + n])
        np.testing.assert_allclose(grid.zero, ref[5:5 + n], rtol=1e-14, atol=1e-16)
    for row, back, wl in zip(g['cn2'], g['r0_back'], g['wavelengths']):
        for r0, c, rb in zip(g['r0'], row, back):
            assert hg.Cn_squared_from_fried_parameter(r0, wl) == pytest.approx(c, rel=1e-14)
            assert hg.fried_parameter_from_Cn_squared(c, wl) == pytest.approx(rb, rel=1e-14)
    psd = hg.power_spectral_density_von_karman(0.12, 22.0)(hg.make_pupil_grid(24, 40.0))
    np.testing.assert_allclose(np.asarray(psd), g['psd'], rtol=1e-13)
    np.testing.assert_allclose(von_karman_covariance(g['cov_r'], 0.12, 22.0), g['cov'], rtol=1e-12)


def test_diffraction_scaled_focal_grids():
    """The broadband workload's per-wavelength focal grids: q = 4 everywhere, the radius num_airy lambda0/lambda,
    so 21 wavelengths over 0.9-1.1 lambda0 give uneven sizes from 284^2 down to 232^2 (1,386,546 pixels)."""
    wls = np.linspace(0.9, 1.1, 21)
    grids = hg.diffraction_scaled_focal_grids(4, 32, wls, 1.0)
    sizes = [int(g.dims[0]) for g in grids]
    assert sizes[0] == 284 and sizes[-1] == 232 and sizes == sorted(sizes, reverse=True)
    assert all(int(g.dims[0]) == int(g.dims[1]) for g in grids)
    assert sum(g.size for g in grids) == 1386546
    for g, wl in zip(grids, wls):
        np.testing.assert_allclose(g.delta, 0.25, rtol=0)
        assert int(g.dims[0]) == int(2 * 4 * 32 / wl)


def test_optical_system_and_empty_element():
    """OpticalSystem (optical_element.py:848-950) applies its elements' forwards in order and their backwards in
    reverse order; EmptyOpticalElement (:153-218) returns the wavefront it is given.  Host logic: the elements
    here record the calls."""
    calls = []

    class Step(hg.OpticalElement):
        def __init__(self, name):
            self.name = name

        def forward(self, wf):
            calls.append(('f', self.name))
            return wf + [self.name]

        def backward(self, wf):
            calls.append(('b', self.name))
            return wf + [self.name.upper()]

    system = hg.OpticalSystem((Step('a'), hg.EmptyOpticalElement(), Step('b')))
    assert isinstance(system.optical_elements, list) and len(system.optical_elements) == 3
    assert system.forward([]) == ['a', 'b'] and system([]) == ['a', 'b']
    assert system.backward([]) == ['B', 'A']
    assert calls == [('f', 'a'), ('f', 'b'), ('f', 'a'), ('f', 'b'), ('b', 'b'), ('b', 'a')]
    token = object()
    assert hg.EmptyOpticalElement().forward(token) is token and hg.EmptyOpticalElement().backward(token) is token
