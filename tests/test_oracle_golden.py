"""Pin the numpy oracle against golden vectors produced by the HCIPy reference itself."""
import numpy as np
import pytest

from conftest import load_golden, grid_from, rel_err
from oracle import fourier, optics, atmosphere, grids


@pytest.mark.parametrize('case', ['mft_0', 'mft_1', 'mft_2'])
def test_mft_oracle(case):
    g = load_golden(case)
    x, y, u, v = g['in_x'], g['in_y'], g['out_x'], g['out_y']
    w_in = g['ingrid_weights'][0]
    w_out = g['outgrid_weights'][0]
    fwd = fourier.mft_forward(g['E'], x, y, u, v, w_in)
    bwd = fourier.mft_backward(g['F'], x, y, u, v, w_out)
    assert rel_err(fwd, g['fwd_c128']) < 1e-13
    assert rel_err(bwd, g['bwd_c128']) < 1e-13
    # The reference's own complex64 result is within single precision of float64.
    assert rel_err(g['fwd_c64'], g['fwd_c128']) < 1e-5


def test_mft1d_oracle():
    g = load_golden('mft_1d')
    fwd = fourier.mft1d_forward(g['E'], g['in_x'], g['out_x'], g['w_in'])
    bwd = fourier.mft1d_backward(g['F'], g['in_x'], g['out_x'], g['w_out'])
    assert rel_err(fwd, g['fwd_c128']) < 1e-13
    assert rel_err(bwd, g['bwd_c128']) < 1e-13


def test_grid_factories():
    g = load_golden('fraunhofer_cfg1')
    pupil = grids.make_pupil_grid(256, 1)
    focal = grids.make_focal_grid(4, 16)
    np.testing.assert_allclose(pupil.delta, g['pupil_delta'], rtol=0, atol=0)
    np.testing.assert_allclose(pupil.zero, g['pupil_zero'], rtol=1e-15)
    np.testing.assert_array_equal(focal.dims, g['focal_dims'])
    np.testing.assert_allclose(focal.zero, g['focal_zero'], rtol=1e-15)


def test_fraunhofer_cfg1_oracle():
    g = load_golden('fraunhofer_cfg1')
    pupil = grid_from(g, 'pupil')
    focal = grid_from(g, 'focal')
    res = optics.fraunhofer_forward(g['E'], pupil, focal)
    assert rel_err(res, g['focal_c128']) < 1e-13
    back = optics.fraunhofer_backward(g['focal_c128'], pupil, focal)
    assert rel_err(back, g['back_c128']) < 1e-13


@pytest.mark.parametrize('case', ['fft_0', 'fft_1', 'fft_2', 'fft_3'])
def test_fft_oracle(case):
    g = load_golden(case)
    pupil = grid_from(g, 'ingrid')
    plan = fourier.FFTPlan(pupil, g['q'], g['fov'], g['shift'])
    np.testing.assert_array_equal(plan.output_grid.dims, g['outgrid_dims'])
    np.testing.assert_allclose(plan.output_grid.zero, g['outgrid_zero'], rtol=1e-12, atol=1e-14)
    fwd = plan.forward(g['E'])
    assert rel_err(fwd, g['fwd_exact_c128']) < 1e-13
    # The reference's default (emulated fftshifts) agrees to float64 round-off.
    assert rel_err(fwd, g['fwd_c128']) < 1e-12
    bwd = plan.backward(g['F'])
    assert rel_err(bwd, g['bwd_c128']) < 1e-12


def test_czt_oracle():
    g = load_golden('czt')
    for i in range(4):
        x, w, a, m = g['x_%d' % i], complex(g['w_%d' % i]), complex(g['a_%d' % i]), int(g['m_%d' % i])
        y = fourier.czt(x, m, w, a)
        assert rel_err(y, g['y_%d' % i]) < 1e-13
        if len(x) <= 128:
            assert rel_err(fourier.czt_direct(x, m, w, a), g['y_%d' % i]) < 1e-10
    yb = fourier.czt(g['xb'], 31, np.exp(-0.2j), np.exp(0.7j))
    assert rel_err(yb, g['yb']) < 1e-13


def test_zoomfft_oracle():
    g = load_golden('zoomfft')
    gi, go = grid_from(g, 'ingrid'), grid_from(g, 'outgrid')
    assert rel_err(fourier.zoomfft_forward(g['E'], gi, go), g['fwd_c128']) < 1e-12
    assert rel_err(fourier.zoomfft_backward(g['F'], gi, go), g['bwd_c128']) < 1e-12
    # ZoomFFT and MFT compute the same transform.
    x, y = gi.separated_coords
    u, v = go.separated_coords
    assert rel_err(fourier.mft_forward(g['E'], x, y, u, v, gi.weights), g['fwd_c128']) < 1e-10


def test_fourier_filter_oracle():
    g = load_golden('fourier_filter')
    gi = grid_from(g, 'ingrid')
    plan = fourier.FourierFilterPlan(gi, g['tf'], q=2)
    assert rel_err(plan.apply(g['E']), g['fwd_c128']) < 1e-13
    assert rel_err(plan.apply(g['E'], adjoint=True), g['bwd_c128']) < 1e-13


@pytest.mark.parametrize('case', ['asp_0', 'asp_1', 'asp_2', 'asp_3'])
def test_asp_oracle(case):
    g = load_golden(case)
    pupil = grids.make_pupil_grid(int(g['n']), float(g['diam']))
    wl, d = float(g['wavelength']), float(g['distance'])
    assert fourier.asp_uses_impulse_branch(pupil, wl, d) == bool(g['impulse_branch'])
    if bool(g['impulse_branch']):
        pytest.skip('impulse-response branch is checked on the device path only')
    internal = grids.make_fft_grid(pupil, 2, 1)
    tf = fourier.asp_transfer_function(internal, wl, d)
    plan = fourier.FourierFilterPlan(pupil, tf, q=2)
    assert rel_err(plan.apply(g['E']), g['fwd_c128']) < 1e-10
    assert rel_err(plan.apply(g['fwd_c128'], adjoint=True), g['bwd_c128']) < 1e-10


@pytest.mark.parametrize('case', ['fresnel_0', 'fresnel_1', 'fresnel_2', 'fresnel_3', 'fresnel_4'])
def test_fresnel_oracle(case):
    """Both branches of the Fresnel transfer function (fresnel.py:45-80) through the Fourier filter with the
    case's zero padding, against the reference's propagation."""
    g = load_golden(case)
    pupil = grids.make_pupil_grid(int(g['n']), float(g['diam']))
    wl, d, q, nref = float(g['wavelength']), float(g['distance']), int(g['zero_padding']), float(g['refractive_index'])
    impulse = fourier.fresnel_uses_impulse_branch(pupil, wl, d)
    assert impulse == bool(g['impulse_branch'])
    internal = grids.make_fft_grid(pupil, q, 1)
    make_tf = fourier.fresnel_impulse_transfer_function if impulse else fourier.fresnel_transfer_function
    plan = fourier.FourierFilterPlan(pupil, make_tf(internal, wl, d, nref), q=q)
    assert rel_err(plan.apply(g['E']), g['fwd_c128']) < 1e-10
    assert rel_err(plan.apply(g['fwd_c128'], adjoint=True), g['bwd_c128']) < 1e-10


def test_lyot_oracle():
    g = load_golden('lyot')
    pupil, fpm_grid, focal = grid_from(g, 'pupil'), grid_from(g, 'fpm'), grid_from(g, 'focal')
    lyot = optics.lyot_forward(g['E'], pupil, fpm_grid, g['fpm'], g['stop'])
    assert rel_err(lyot, g['lyot_c128']) < 1e-11
    img = optics.fraunhofer_forward(lyot, pupil, focal)
    assert rel_err(img, g['image_c128']) < 1e-10
    # Wavefront.power = |E|^2 * weights (hcipy/optics/wavefront.py:341-357).
    peak = np.max(np.abs(optics.fraunhofer_forward(g['aperture'], pupil, focal))**2) * focal.weights
    assert abs(peak / g['ref_peak'] - 1) < 1e-12


def test_subpixel_oracle():
    g = load_golden('subpixel')
    for i in range(4):
        dy, dx = float(g['dy_%d' % i]), float(g['dx_%d' % i])
        np.testing.assert_allclose(atmosphere.quintic_weights(dy), g['wy_%d' % i], rtol=0, atol=1e-15)
        out = atmosphere.subpixel_shift(g['img'], dy, dx)
        np.testing.assert_allclose(out, g['out_%d' % i], rtol=1e-12, atol=1e-13)
    with pytest.raises(ValueError):
        atmosphere.subpixel_shift(g['img'], 0.6, 0)


def test_atmosphere_replay_oracle():
    g = load_golden('atmosphere')
    pupil = grid_from(g, 'pupil')
    shape = pupil.shape
    screen = g['screen0']
    center = np.zeros(2)
    t = 0.0
    for i in range(3):
        dt = float(g['dt_%d' % i])
        center, steps, sub = atmosphere.evolve_steps(center, g['velocity'], t, t + dt, pupil.delta)
        t += dt
        noise = g['noise_%d' % i]
        assert noise.shape[0] == abs(steps[0])
        for k in range(abs(steps[0])):
            where = 'left' if steps[0] < 0 else 'right'
            screen = atmosphere.extrude(screen, shape, where, g['A_horizontal'], g['B_horizontal'], g['stencil_left_idx'], noise[k])
        np.testing.assert_allclose(screen, g['screen_%d' % i], rtol=1e-12, atol=1e-15)
        shifted = atmosphere.subpixel_shift(screen.reshape(shape), sub[1] / pupil.delta[1], sub[0] / pupil.delta[0])
        np.testing.assert_allclose(shifted.ravel(), g['shifted_%d' % i], rtol=1e-12, atol=1e-15)


def test_dm_oracle():
    g = load_golden('dm')
    surf = optics.dm_surface(g['influence'], g['actuators'])
    np.testing.assert_allclose(surf, g['surface'], rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(optics.dm_forward(g['E'], surf, 1.0), g['fwd_c128'], rtol=1e-12, atol=1e-14)


def test_efc_oracle():
    """The regularised inverses and the tutorial's poke Jacobian / EFC loop, restated in numpy, against the
    reference run on the same seeded 32^2 case."""
    from oracle import efc
    g = load_golden('efc')
    m = g['M']
    assert rel_err(efc.inverse_tikhonov(m, 1e-3), g['M_tikhonov']) < 1e-10
    assert rel_err(efc.inverse_truncated(m, 1e-4), g['M_truncated']) < 1e-10
    assert rel_err(efc.inverse_truncated_modal(m, 5), g['M_modal']) < 1e-10
    pupil, fpm_grid, focal = grid_from(g, 'pupil'), grid_from(g, 'fpm'), grid_from(g, 'focal')
    inf, dz = g['influence'], g['dark_zone']

    def field(act, e):
        e = optics.dm_forward(e, inf @ act, 1.0)
        return optics.fraunhofer_forward(optics.lyot_forward(e, pupil, fpm_grid, g['fpm'], g['stop']), pupil, focal)

    jac = efc.poke_jacobian(lambda c: field(c, g['aperture'].astype(complex)), dz, inf.shape[1], g['epsilon'])
    assert rel_err(jac, g['jacobian']) < 1e-8
    em = efc.inverse_tikhonov(g['jacobian'], g['rcond'])
    assert rel_err(em, g['efc_matrix']) < 1e-10
    act = g['actuators'][0]
    for k in range(1, len(g['actuators'])):
        act = efc.efc_step(em, field(act, g['aberration']), dz, act, g['gain'])
        assert rel_err(act, g['actuators'][k]) < 1e-9


def test_spectral_noise_oracle():
    """Multi-scale spectral noise with the von Karman PSD (hcipy/util/spectral_noise.py:203-320): the seeded
    realization and its shifted evaluation, as the reference drew them."""
    g = load_golden('spectral_noise')
    grid = grid_from(g, 'grid')
    rng = np.random.default_rng(int(g['seed']))
    s = atmosphere.multiscale_spectral_noise(grid, float(g['r0']), float(g['L0']), int(g['oversampling']), rng)
    assert rel_err(s, g['screen']) < 1e-12
    rng = np.random.default_rng(int(g['seed']))
    s = atmosphere.multiscale_spectral_noise(grid, float(g['r0']), float(g['L0']), int(g['oversampling']), rng,
                                             shift=g['shift'])
    assert rel_err(s, g['shifted']) < 1e-12


def test_infinite_layer_initial_screen_oracle():
    """A seeded infinite layer's initial screen is multi-scale spectral noise at oversampling 16 drawn from the
    layer's generator after its stencil draws (infinite_atmospheric_layer.py:111-140, 204-214), and the first
    extrusion's noise continues that generator."""
    g = load_golden('atmosphere')
    grid = grid_from(g, 'pupil')
    nx, ny = (int(d) for d in g['pupil_dims'])
    rng = np.random.default_rng(5)
    rng.geometric(0.5, nx)
    rng.geometric(0.5, ny)
    r0 = (0.423 * float(g['cn2']) * (2 * np.pi)**2)**(-3. / 5)  # Fried parameter at a wavelength of 1 m
    screen = atmosphere.multiscale_spectral_noise(grid, r0, 25.0, 16, rng)
    assert rel_err(screen, g['screen0']) < 1e-12
    noise = rng.normal(0, np.sqrt(float(g['cn2'])), size=g['noise_0'].shape[1])
    assert np.array_equal(noise, g['noise_0'][0])


def _pyramid_optics(pupil_n, wfs_n):
    return optics.PyramidOptics(grids.make_pupil_grid(pupil_n, 1.0), grids.make_pupil_grid(wfs_n, 2.0), 1.0, 1.0, 1.0,
                                lambda wl: 1.5 + 0.01 * (wl - 1.0))


def test_pyramid_oracle():
    """The pyramid optics (hcipy/wavefront_sensing/pyramid.py:94-181) at two wavelengths of a dispersive glass."""
    g = load_golden('pyramid')
    po = _pyramid_optics(48, 96)
    np.testing.assert_array_equal(po.focal.dims, g['focal_dims'])
    for k in range(2):
        assert rel_err(po.forward(g['E'], float(g['wavelength_%d' % k])), g['fwd_%d' % k]) < 1e-12, k


def test_modulated_pyramid_oracle():
    """The modulated pyramid (pyramid.py:10-91): both methods, the shifted pyramid's supersampled sag bit for bit,
    and the tip-tilt mirror (hcipy/optics/tip_tilt_mirror.py)."""
    g = load_golden('modulated_pyramid')
    po = _pyramid_optics(32, 40)
    mod, steps = float(g['modulation']), int(g['num_steps'])
    assert np.array_equal(optics.modulation_positions(mod, steps), g['positions'])
    assert rel_err(optics.modulated_pyramid_forward(po, g['E'], 1.0, mod, steps), g['slow']) < 1e-12
    for k in range(2):
        out = optics.modulated_pyramid_forward(po, g['E'], float(g['wavelength_%d' % k]), mod, steps, fast=True)
        assert rel_err(out, g['fast_%d' % k]) < 1e-12, k
    sag = fourier.supersampled_mean(po.sag_function, po.focal.shifted(2 * g['positions'][3]), 4)
    assert np.array_equal(sag, g['fast_surface_3'])
    pupil = grids.make_pupil_grid(32, 1.0)
    assert rel_err(optics.tip_tilt_forward(g['E'], pupil, g['tip_tilt_command'], 0.8), g['tip_tilt']) < 1e-14


@pytest.mark.parametrize('case', ['vortex_0', 'vortex_1'])
def test_vortex_oracle(case):
    """The multi-scale vortex (hcipy/coronagraphy/multi_scale.py, vortex.py:12-15): level masks, Lyot plane and
    backward propagation."""
    g = load_golden(case)
    ms = optics.MultiScaleOptics(grids.make_pupil_grid(int(g['n']), 1.0), optics.vortex_mask(int(g['charge'])),
                                 int(g['q']), int(g['scaling_factor']), int(g['window_size']))
    assert len(ms.masks) == int(g['levels'])
    for k, m in enumerate(ms.masks):
        assert rel_err(m, g['mask_%d' % k]) < 1e-12, k
    assert rel_err(ms.propagate(g['E']), g['lyot_c128']) < 1e-12
    assert rel_err(ms.propagate(g['G'], adjoint=True), g['back_c128']) < 1e-12


def test_vector_vortex_oracle():
    """The vector vortex (vortex.py:17-246) in the reference's own tensor form (a Jones-matrix transfer function and
    field_dot at every level), and the Stokes parameters of a partially polarised wavefront (wavefront.py:103-235)
    through the Mueller matrix."""
    g = load_golden('vector_vortex')
    pupil = grids.make_pupil_grid(48, 1.0)
    focal = grids.make_focal_grid(4, 8)
    stop = g['stop']
    for k in range(2):
        wl = float(g['wavelength_%d' % k])
        vv = optics.MultiScaleOptics(pupil, optics.vector_vortex_mask(2, np.pi * (1 + 0.05 * (wl - 1))), 32, 2, 16)
        lyot = vv.propagate(g['E']) * stop
        assert rel_err(lyot, g['lyot_%d' % k]) < 1e-12, k
        img = np.array([[optics.fraunhofer_forward(lyot[i, j], pupil, focal, wavelength=wl) for j in range(2)]
                        for i in range(2)])
        assert rel_err(optics.stokes_parameters(img, g['lyot_stokes_%d' % k]), g['image_%d' % k]) < 1e-12, k
    vv = optics.MultiScaleOptics(pupil, optics.vector_vortex_mask(2, np.pi), 32, 2, 16)
    assert rel_err(vv.propagate(g['EJ']) * stop, g['lyot_pol']) < 1e-12
    assert rel_err(optics.stokes_parameters(g['lyot_pol'], g['stokes']), g['lyot_pol_stokes']) < 1e-13
    assert rel_err(vv.propagate(g['G'] * stop, adjoint=True), g['back']) < 1e-12
    assert rel_err(vv.propagate(g['G'][0, 0] * stop, adjoint=True), g['back_scalar']) < 1e-12
