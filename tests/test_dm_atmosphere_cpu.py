"""Host-side plan data of the deformable mirror and the atmospheric layer against the reference's own values.

These run without a GPU: the influence functions, the extrusion stencils and the autoregressive matrices are
built on the host (as the reference builds them), so they are compared with the golden vectors directly.
Tolerances: the same float64 operations in the same order as the reference, so 1e-12 relative (observed 0).
"""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytest.importorskip('scipy')


def _grid(rec, prefix):
    from hcipy_gb300.field import CartesianGrid, RegularCoords
    return CartesianGrid(RegularCoords(rec[prefix + '_delta'], rec[prefix + '_dims'], rec[prefix + '_zero']))


def test_gaussian_influence_functions_match_reference():
    from hcipy_gb300 import deformable_mirror as dmm
    g = load_golden('dm')
    inf = dmm.make_gaussian_influence_functions(_grid(g, 'pupil'), 8, 1 / 8, crosstalk=0.15)
    m = inf.transformation_matrix.toarray()
    assert m.shape == g['influence'].shape
    assert np.count_nonzero(m) == np.count_nonzero(g['influence'])
    assert rel_err(m, g['influence']) < 1e-12
    assert rel_err(m @ g['actuators'], g['surface']) < 1e-12


def test_find_illuminated_actuators():
    from hcipy_gb300 import deformable_mirror as dmm
    g = load_golden('dm')
    grid = _grid(g, 'pupil')
    inf = dmm.make_gaussian_influence_functions(grid, 8, 1 / 8, crosstalk=0.15)
    aperture = np.abs(g['E']) > 0
    sel = dmm.find_illuminated_actuators(inf, aperture, 0.1)
    m = g['influence']
    keep = (np.abs(m[aperture])**2).sum(0) >= 0.1 * (np.abs(m)**2).sum(0)
    assert sel.num_modes == keep.sum()
    assert rel_err(sel.transformation_matrix.toarray(), m[:, keep]) < 1e-12


def test_actuator_positions_bmc_convention():
    from hcipy_gb300.deformable_mirror import make_actuator_positions
    x, y = make_actuator_positions(4, 0.25)
    assert np.allclose(np.unique(x), [-0.375, -0.125, 0.125, 0.375])
    assert np.allclose(np.unique(y), [-0.375, -0.125, 0.125, 0.375])


def test_atmosphere_stencils_and_matrices_match_reference():
    from hcipy_gb300 import atmosphere as at
    g = load_golden('atmosphere')
    grid = _grid(g, 'pupil')
    nx, ny = (int(d) for d in g['pupil_dims'])
    bottom, left = at.make_stencils(nx, ny, 2, np.random.default_rng(5))
    assert np.array_equal(bottom, g['stencil_bottom_idx'])
    assert np.array_equal(left, g['stencil_left_idx'])
    av, bv = at.ar_matrices(grid, bottom, 'bottom', 25)
    ah, bh = at.ar_matrices(grid, left, 'left', 25)
    assert rel_err(av, g['A_vertical']) < 1e-12
    assert rel_err(ah, g['A_horizontal']) < 1e-12
    # B is defined up to the signs of the singular vectors: compare B B^T, and B itself (same LAPACK here).
    assert rel_err(bv @ bv.T, g['B_vertical'] @ g['B_vertical'].T) < 1e-12
    assert rel_err(bh @ bh.T, g['B_horizontal'] @ g['B_horizontal'].T) < 1e-12


def test_quintic_weights_match_reference():
    from hcipy_gb300.atmosphere import quintic_weights
    g = load_golden('subpixel')
    for i in range(4):
        assert rel_err(quintic_weights(float(g['dy_%d' % i])), g['wy_%d' % i]) < 1e-14
        assert rel_err(quintic_weights(float(g['dx_%d' % i])), g['wx_%d' % i]) < 1e-14


def test_von_karman_screen_statistics():
    """The package's initial screen follows the von Karman structure function 2 (C(0) - C(r)) within the
    sampling error and the power lost above the grid's Nyquist frequency (10-15% at 4-8 pixels)."""
    from hcipy_gb300 import atmosphere as at
    rng = np.random.default_rng(0)
    n, d, l0 = 128, 8.0 / 128, 25.0
    cn2 = at.Cn_squared_from_fried_parameter(0.5, 500e-9)
    r0 = at.fried_parameter_from_Cn_squared(cn2, 1.0)
    for lag in (4, 8):
        sf = []
        for _ in range(6):
            s = at.von_karman_screen(n, n, np.array([d, d]), cn2, l0, rng, pad=4)
            sf.append(np.mean((s[:, lag:] - s[:, :-lag])**2))
        theory = 2 * (at.von_karman_covariance(0.0, r0, l0) - at.von_karman_covariance(lag * d, r0, l0))
        assert 0.75 < np.mean(sf) / theory < 1.1, (lag, np.mean(sf) / theory)


def test_oracle_lyot_adjoint_and_gradient():
    """The oracle's adjoint chain (the checker of the device gradients): dot-product identity and central
    differences of its loss."""
    import hcipy_gb300 as hg
    from hcipy_gb300 import workloads
    from hcipy_gb300.deformable_mirror import make_gaussian_influence_functions
    from oracle import optics as oo
    from oracle.grids import RegularGrid
    og = lambda g: RegularGrid(g.delta, g.dims, g.zero)  # noqa: E731
    pupil, fpm_grid, focal = hg.make_pupil_grid(48, 1), hg.make_focal_grid(3.7, 6), hg.make_focal_grid(3.3, 8)
    fpm = 1 - workloads.circular_aperture(fpm_grid, 5.0)
    ch = oo.LyotChain(og(pupil), og(fpm_grid), og(focal), fpm, workloads.circular_aperture(pupil, 0.9))
    rng = np.random.default_rng(0)
    x = rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)
    w = rng.standard_normal(focal.size) + 1j * rng.standard_normal(focal.size)
    lhs, rhs = np.vdot(w, ch(x)), np.vdot(ch.lyot_adjoint(ch.image_adjoint(w)), x)
    assert abs(lhs - rhs) < 1e-13 * np.linalg.norm(w) * np.linalg.norm(ch(x))
    inf = make_gaussian_influence_functions(pupil, 6, 1 / 6).transformation_matrix
    ap = workloads.circular_aperture(pupil, 1.0)
    fx, fy = focal.points_list()
    roi = (np.hypot(fx, fy) >= 2) & (np.hypot(fx, fy) <= 6) & (fx > 0)
    a = rng.standard_normal(inf.shape[1]) * 2e-3
    _, g = oo.dm_lyot_loss_grad(ch, inf, ap, a, roi)
    h = 1e-6
    for i in (3, 7, 20):
        ap_, am_ = a.copy(), a.copy()
        ap_[i] += h
        am_[i] -= h
        fd = (oo.dm_lyot_loss_grad(ch, inf, ap, ap_, roi)[0] - oo.dm_lyot_loss_grad(ch, inf, ap, am_, roi)[0]) / (2 * h)
        assert abs(fd - g[i]) < 1e-7 * np.abs(g).max()


def test_scintillation_element_order():
    """The scintillating multi-layer sequence (atmospheric_model.py:185-212): layers from the highest down, a
    Fresnel propagation over each height difference, and one to the ground when the lowest layer is above it."""
    import hcipy_gb300 as hg

    class Stub(object):
        def __init__(self, h):
            self.height = h
            self.input_grid = hg.make_pupil_grid(8, 1.0)

    a, b, c = Stub(5000.0), Stub(0.0), Stub(2000.0)
    els = hg.MultiLayerAtmosphere([a, b, c], scintillation=True).calculate_propagators()
    assert els[0] is a and els[2] is c and els[4] is b and len(els) == 5
    assert [e.distance for e in (els[1], els[3])] == [3000.0, 2000.0]
    assert all(isinstance(e, hg.FresnelPropagator) for e in (els[1], els[3]))
    els = hg.MultiLayerAtmosphere([Stub(300.0), Stub(1000.0)], scintillation=True).calculate_propagators()
    assert [getattr(e, 'distance', None) for e in els] == [None, 700.0, None, 300.0]


@pytest.mark.parametrize('block', [4, 3])
def test_actuator_block_lists_reproduce_the_transpose(block):
    """The plan-time union lists of the blocked DM transpose (blocks of consecutive actuators, the union of their
    pixels, one weight per actuator of the block and zero where it does not reach): summing weight x gradient
    over every list in numpy gives M^T g exactly as the CSC product does, for a ragged last block, empty columns
    and a Gaussian-influence basis."""
    import scipy.sparse as sp
    import hcipy_gb300 as hg
    from hcipy_gb300.kernels import _actuator_blocks
    rng = np.random.default_rng(block)
    grid = hg.make_pupil_grid(48, 1)
    gauss = sp.csc_matrix(hg.make_gaussian_influence_functions(grid, 7, 1 / 7).transformation_matrix)
    rand = sp.random(500, 23, density=0.1, random_state=3, format='lil')
    rand[:, 5] = 0  # an actuator that reaches no pixel
    rand = sp.csc_matrix(rand)
    rand.eliminate_zeros()
    for m in (gauss, rand):
        m.sort_indices()
        ptr, pix, vals = _actuator_blocks(m, block)
        vals = vals.reshape(-1, block)
        nact = m.shape[1]
        assert ptr.size == -(-nact // block) + 1 and ptr[-1] == pix.size == vals.shape[0]
        g = rng.standard_normal((3, m.shape[0]))
        out = np.zeros((3, nact))
        for b in range(ptr.size - 1):
            seg = slice(ptr[b], ptr[b + 1])
            assert np.all(np.diff(pix[seg]) > 0)  # sorted, no repeats
            for q in range(block):
                a = b * block + q
                if a < nact:
                    out[:, a] = g[:, pix[seg]] @ vals[seg, q]
        np.testing.assert_allclose(out, g @ m.toarray(), rtol=1e-12, atol=1e-12)


def test_broadband_phase_screen_hook_resolution():
    """BroadbandImager fuses the phase of ``pre`` only when ``pre`` is a pure phase element: the element itself or
    its bound ``forward``; any other callable keeps the separate phase application (host logic)."""
    import hcipy_gb300 as hg

    class Screen(object):
        def __init__(self):
            self.calls = 0

        def forward(self, wf):
            return wf

        __call__ = forward

        def _pure_phase_screen(self):
            self.calls += 1
            return 'screen'

    s = Screen()
    pupil = hg.make_pupil_grid(16, 1)
    grids = [hg.make_focal_grid(2, 4)]
    for pre, expect in ((s, 'screen'), (s.forward, 'screen'), (lambda wf: s.forward(wf), None), (None, None)):
        imager = hg.BroadbandImager(pupil, [1.0], grids, pre=pre)
        assert imager._phase_screen() == expect


def test_modulated_pyramid_plan_time_host_data():
    """The modulated pyramid's plan-time data, built on the host: the modulation positions and the shifted
    pyramid's supersampled sags equal the reference's bit for bit; the tip-tilt mirror's modes are the grid's x
    and y; backward is refused as in the reference."""
    import hcipy_gb300 as hg
    g = load_golden('modulated_pyramid')
    pupil = hg.make_pupil_grid(32, 1.0)
    pwfs = hg.PyramidWavefrontSensorOptics(pupil, hg.make_pupil_grid(40, 2.0), separation=1.0, pupil_diameter=1.0,
                                           wavelength_0=1.0, refractive_index=lambda wl: 1.5 + 0.01 * (wl - 1.0))
    mod = hg.ModulatedPyramidWavefrontSensorOptics(pwfs, float(g['modulation']), num_steps=int(g['num_steps']),
                                                   fast_modulation_method=True)
    assert np.array_equal(mod.modulation_positions.points, g['positions'])
    assert np.array_equal(mod._sags[3], g['fast_surface_3'])
    assert mod._sags.shape == (int(g['num_steps']), pwfs.focal_grid.size)
    slow = hg.ModulatedPyramidWavefrontSensorOptics(pwfs, 3.0, num_steps=5)
    assert slow._sags is None and len(slow.modulation_positions.points) == 5
    m = slow.tip_tilt_mirror.influence_functions.transformation_matrix
    assert np.array_equal(m[:, 0], pupil.x) and np.array_equal(m[:, 1], pupil.y)
    with pytest.raises(RuntimeError):
        slow.backward(None)


def test_vector_vortex_jones_entries():
    """The vector vortex's focal-plane masks (host plan data): the three entries form the Jones matrix of a linear
    retarder R(-a) diag(e^{iG/2}, e^{-iG/2}) R(a) with fast axis a = charge theta / 2 (symmetric and unitary), and
    all vanish at the singularity."""
    import hcipy_gb300 as hg
    grid = hg.make_uniform_grid([9, 9], [2.0, 2.0])  # odd: a point on the singularity
    vvc = hg.VectorVortexCoronagraph(4, phase_retardation=0.9 * np.pi)
    j11, j12, j22 = (vvc._jones_entry(0.9 * np.pi, w)(grid) for w in ('j11', 'j12', 'j22'))
    x, y = grid.points_list()
    a = 2 * np.arctan2(y, x)
    centre = np.hypot(x, y) == 0
    assert centre.sum() == 1 and j11[centre] == 0 and j12[centre] == 0 and j22[centre] == 0
    for k in np.flatnonzero(~centre):
        c, s = np.cos(a[k]), np.sin(a[k])
        rot = np.array([[c, s], [-s, c]])
        ref = rot.T @ np.diag([np.exp(0.45j * np.pi), np.exp(-0.45j * np.pi)]) @ rot
        got = np.array([[j11[k], j12[k]], [j12[k], j22[k]]])
        assert np.allclose(got, ref, rtol=0, atol=1e-15)
        assert np.allclose(got @ got.conj().T, np.eye(2), rtol=0, atol=1e-15)


def test_gaussian_influence_functions_sweep():
    """Gaussian influence functions with other crosstalk and cutoff values, x/y/z-tilted mirrors and oversampled
    evaluation (deformable_mirror.py:43-93) against the reference: the same nonzero pattern and values within
    1e-15 (the reference evaluates the tilted and oversampled grids in another order)."""
    import scipy.sparse
    import hcipy_gb300 as hg
    g = load_golden('influence_sweep')
    pupil = hg.make_pupil_grid(24, 1.0)
    for i in range(int(g['count'])):
        kw = {k: float(g['%s_%d' % (k, i)]) for k in ('crosstalk', 'cutoff', 'x_tilt', 'y_tilt', 'z_tilt')}
        kw['oversampling'] = int(g['oversampling_%d' % i])
        ref = scipy.sparse.csr_matrix((g['data_%d' % i], g['indices_%d' % i], g['indptr_%d' % i]),
                                      shape=tuple(g['shape_%d' % i])).toarray()
        mine = hg.make_gaussian_influence_functions(pupil, 5, 1 / 5, **kw).transformation_matrix.toarray()
        assert np.array_equal(mine != 0, ref != 0), i
        assert np.max(np.abs(mine - ref)) < 1e-15, (i, kw)


def test_atmosphere_matrices_for_other_layers():
    """Stencils and autoregressive matrices (infinite_atmospheric_layer.py:111-202) of a rectangular grid and of a
    longer stencil with another outer scale against the reference: the same stencil draws, A within 1e-12, and
    B B^T within 1e-12 (B is defined up to the signs of its singular vectors)."""
    from hcipy_gb300 import atmosphere as at
    from hcipy_gb300.field import CartesianGrid, RegularCoords
    g = load_golden('atmosphere_matrices')
    for i in range(int(g['count'])):
        grid = CartesianGrid(RegularCoords(g['delta_%d' % i], g['dims_%d' % i], g['zero_%d' % i]))
        nx, ny = (int(d) for d in g['dims_%d' % i])
        bottom, left = at.make_stencils(nx, ny, int(g['stencil_length_%d' % i]),
                                        np.random.default_rng(int(g['seed_%d' % i])))
        assert np.array_equal(bottom, g['stencil_bottom_%d' % i]) and np.array_equal(left, g['stencil_left_%d' % i])
        for where, stencil, key in (('bottom', bottom, 'vertical'), ('left', left, 'horizontal')):
            a, b = at.ar_matrices(grid, stencil, where, float(g['L0_%d' % i]))
            assert rel_err(a, g['A_%s_%d' % (key, i)]) < 1e-12, (i, key)
            ref_b = g['B_%s_%d' % (key, i)]
            assert rel_err(b @ b.T, ref_b @ ref_b.T) < 1e-12, (i, key)
