"""Infinite atmospheric layer and sub-pixel shift on the GPU against the reference's replayed values.

The golden case is the reference's own layer (24^2 grid, seed 5, L0 = 25 m, wind along x) evolved over three
time steps; the layer here starts from the reference's initial screen, uses the reference's A and B matrices
(B comes from an SVD whose singular vectors differ between LAPACK builds at ~1e-9; the host-side matrices are
pinned separately on the CPU) and is fed the reference's noise rows, so every extruded column and every
sub-pixel-shifted screen must agree.
Tolerances: float64 screens 1e-12 relative (the same products summed in another order); float32 1e-5.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def _grid(rec, prefix):
    return hg.CartesianGrid(hg.RegularCoords(rec[prefix + '_delta'], rec[prefix + '_dims'], rec[prefix + '_zero']))


def _use_reference_matrices(layer, g):
    layer.A_vertical, layer.B_vertical = g['A_vertical'], g['B_vertical']
    layer.A_horizontal, layer.B_horizontal = g['A_horizontal'], g['B_horizontal']
    layer._upload_matrices()


class _Replay(object):
    """Stands in for the layer's generator: returns the recorded extrusion noise rows in order."""

    def __init__(self, rows):
        self.rows = list(rows)

    def normal(self, loc, scale, size):
        return self.rows.pop(0)


def test_subpixel_shift_matches_reference():
    g = load_golden('subpixel')
    for i in range(4):
        out = hg.subpixel_shift(torch.from_numpy(g['img']), float(g['dy_%d' % i]), float(g['dx_%d' % i]))
        assert rel_err(out.cpu().numpy(), g['out_%d' % i]) < 1e-13
    with pytest.raises(ValueError):
        hg.subpixel_shift(torch.from_numpy(g['img']), 0.6, 0.0)


@pytest.mark.parametrize('dtype,tol', [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_infinite_layer_replays_reference(dtype, tol):
    g = load_golden('atmosphere')
    grid = _grid(g, 'pupil')
    layer = hg.InfiniteAtmosphericLayer(grid, float(g['cn2']), L0=25, velocity=tuple(g['velocity']),
                                        use_interpolation=True, seed=5, dtype=dtype, initial_screen=g['screen0'])
    assert np.array_equal(layer.stencil_bottom_idx, g['stencil_bottom_idx'])
    _use_reference_matrices(layer, g)
    rows = [r for i in range(3) for r in g['noise_%d' % i]]
    layer.rng = _Replay(rows)
    t = 0.0
    for i in range(3):
        t += float(g['dt_%d' % i])
        layer.t = t
        assert rel_err(layer.achromatic_screen.numpy(), g['screen_%d' % i]) < tol, i
        assert rel_err(layer.phase_for(1.0).numpy(), g['shifted_%d' % i]) < tol, i
    assert not layer.rng.rows


def test_layer_extrudes_all_four_directions_like_the_oracle():
    """Bottom/top/left/right extrusions through the ring buffer against the oracle's array copies."""
    from oracle import atmosphere as oatm
    g = load_golden('atmosphere')
    grid = _grid(g, 'pupil')
    nx, ny = (int(d) for d in g['pupil_dims'])
    layer = hg.InfiniteAtmosphericLayer(grid, float(g['cn2']), L0=25, seed=5, initial_screen=g['screen0'])
    _use_reference_matrices(layer, g)
    rng = np.random.default_rng(9)
    screen = g['screen0'].copy()
    # the ring has a spare row and column: runs of 30 steps wrap both offsets past the ends
    for where in ['right', 'top', 'left', 'bottom', 'top', 'right', 'right', 'bottom'] + ['left'] * 30 + \
            ['top'] * 30 + ['right'] * 3 + ['bottom'] * 31:
        vertical = where in ('top', 'bottom')
        a = g['A_vertical'] if vertical else g['A_horizontal']
        b = g['B_vertical'] if vertical else g['B_horizontal']
        idx = g['stencil_bottom_idx'] if vertical else g['stencil_left_idx']
        noise = rng.standard_normal(b.shape[1])
        screen = oatm.extrude(screen, (ny, nx), where, a, b, idx, noise)
        layer._extrude(where, torch.from_numpy(noise).cuda())
        assert rel_err(layer.achromatic_screen.numpy(), screen) < 1e-12, where


def test_layer_forward_backward_and_multilayer():
    g = load_golden('atmosphere')
    grid = _grid(g, 'pupil')
    l1 = hg.InfiniteAtmosphericLayer(grid, float(g['cn2']), L0=25, velocity=3.0, seed=5, initial_screen=g['screen0'])
    l2 = hg.InfiniteAtmosphericLayer(grid, float(g['cn2']) * 2, L0=25, velocity=(0.0, -2.0), seed=6)
    atm = hg.MultiLayerAtmosphere([l1, l2])
    atm.evolve_until(0.05)
    wl = 0.7
    rng = np.random.default_rng(0)
    e = rng.standard_normal(grid.size) + 1j * rng.standard_normal(grid.size)
    wf = hg.Wavefront(hg.Field(e, grid), wl)
    phase = l1.phase_for(wl).numpy() + l2.phase_for(wl).numpy()
    assert rel_err(atm.phase_for(wl).numpy(), phase) < 1e-13
    out = atm.forward(wf).electric_field.numpy()
    assert rel_err(out, e * np.exp(1j * phase)) < 1e-12
    back = atm.backward(atm.forward(wf)).electric_field.numpy()
    assert rel_err(back, e) < 1e-12
    with pytest.raises(ValueError):
        l1.evolve_until(0.01)


def test_layer_full_size_extrusion_matches_oracle():
    """A 1024^2 layer (the broadband workload's size): four extrusions in float64 against the oracle's array
    copies with the layer's own matrices and noise."""
    from oracle import atmosphere as oatm
    pupil = hg.make_pupil_grid(1024, 8.0)
    layer = hg.InfiniteAtmosphericLayer(pupil, hg.Cn_squared_from_fried_parameter(0.1, 500e-9), L0=25,
                                        velocity=25.0, seed=5)
    screen = layer.achromatic_screen.numpy()
    rng = np.random.default_rng(3)
    for where in ('right', 'right', 'top', 'left'):
        vertical = where in ('top', 'bottom')
        a = layer.A_vertical if vertical else layer.A_horizontal
        b = layer.B_vertical if vertical else layer.B_horizontal
        idx = layer.stencil_bottom_idx if vertical else layer.stencil_left_idx
        noise = rng.standard_normal(b.shape[1]) * np.sqrt(layer.Cn_squared)
        screen = oatm.extrude(screen, (1024, 1024), where, a, b, idx, noise)
        layer._extrude(where, torch.from_numpy(noise).cuda())
    assert rel_err(layer.achromatic_screen.numpy(), screen) < 1e-12


class _StaticLayer(hg.AtmosphericLayer):
    """A layer whose screen is a fixed device tensor (radians at 1 m)."""

    def __init__(self, grid, screen):
        hg.AtmosphericLayer.__init__(self, grid, 1.0)
        self._s = screen

    def _screen_tensor(self):
        return self._s


def test_multilayer_combined_screen_sums_the_layers():
    """hx_atmosphere_combine: three screens summed in layer order equal torch's left-to-right sum exactly; ten
    screens take two launches (8, then 2 more plus the running sum) and agree to rounding; float64 too."""
    grid = hg.make_pupil_grid(40, 1.0)
    gen = torch.Generator(device='cuda').manual_seed(4)
    for dtype in (torch.float32, torch.float64):
        s = [torch.randn(grid.size, device='cuda', dtype=dtype, generator=gen) for _ in range(10)]
        atm3 = hg.MultiLayerAtmosphere([_StaticLayer(grid, x) for x in s[:3]])
        assert torch.equal(atm3.combined_screen(), s[0] + s[1] + s[2])
        atm10 = hg.MultiLayerAtmosphere([_StaticLayer(grid, x) for x in s])
        ref = torch.stack(s).double().sum(0)
        tol = 1e-6 if dtype == torch.float32 else 1e-14
        assert rel_err(atm10.combined_screen().double().cpu().numpy(), ref.cpu().numpy()) < tol
    odd = hg.make_pupil_grid(13, 1.0)  # 169 values: the last thread takes the scalar tail
    s = [torch.randn(odd.size, device='cuda', generator=gen) for _ in range(2)]
    assert torch.equal(hg.MultiLayerAtmosphere([_StaticLayer(odd, x) for x in s]).combined_screen(), s[0] + s[1])


def test_multilayer_float32_forward_and_tracking():
    """Three float32 infinite layers: one phase application of the summed screen equals the reference's
    layer-by-layer products to float32 rounding of the phase; the sum follows a layer evolved on its own and
    keeps its address (a captured graph stays valid), also across reset()."""
    grid = hg.make_pupil_grid(48, 2.0)
    layers = [hg.InfiniteAtmosphericLayer(grid, hg.Cn_squared_from_fried_parameter(r0, 500e-9), L0=20,
                                          velocity=v, seed=7 + i, dtype=torch.float32)
              for i, (r0, v) in enumerate(((0.1, (10.0, 0.0)), (0.2, (-7.5, 13.0)), (0.3, (-12.5, -21.7))))]
    atm = hg.MultiLayerAtmosphere(layers)
    atm.evolve_until(0.01)
    wl = 700e-9
    rng = np.random.default_rng(2)
    e = (rng.standard_normal(grid.size) + 1j * rng.standard_normal(grid.size)).astype(np.complex64)
    wf = hg.Wavefront(hg.Field(torch.from_numpy(e).cuda(), grid), wl)
    seq = wf
    for layer in layers:
        seq = layer.forward(seq)
    out = atm.forward(wf).electric_field.numpy()
    phase = sum(layer.phase_for(wl).numpy().astype(np.float64) for layer in layers)
    assert np.max(np.abs(phase)) > 1.0  # a phase large enough for its rounding to show
    assert rel_err(out, seq.electric_field.numpy()) < 2e-5
    assert rel_err(out, e * np.exp(1j * phase)) < 2e-5
    buf = atm.combined_screen()
    before = buf.clone()
    layers[2].evolve_until(0.03)
    after = atm.combined_screen()
    assert after.data_ptr() == buf.data_ptr() and not torch.equal(after, before)
    expect = layers[0]._screen_tensor() + layers[1]._screen_tensor() + layers[2]._screen_tensor()
    assert torch.equal(after, expect)
    ptrs = [layer._shifted.data_ptr() for layer in layers]
    atm.reset()
    assert [layer._shifted.data_ptr() for layer in layers] == ptrs
    assert atm.combined_screen().data_ptr() == buf.data_ptr()


def test_multilayer_scintillation_matches_oracle_chain():
    """scintillation=True: layers from the highest down with Fresnel propagation over each height difference
    (atmospheric_model.py:185-212), against the oracle's phase screens and Fresnel filters, forward and backward."""
    from oracle import fourier as ofourier
    from oracle import grids as ogrids
    grid = hg.make_pupil_grid(64, 1.0)
    rng = np.random.default_rng(12)
    wl = 1e-6
    screens = [rng.standard_normal(grid.size) * 2e-7 for _ in range(3)]
    heights = [5000.0, 0.0, 2000.0]
    layers = []
    for s, h in zip(screens, heights):
        layer = _StaticLayer(grid, torch.from_numpy(s).cuda())
        layer.height = h
        layers.append(layer)
    atm = hg.MultiLayerAtmosphere(layers, scintillation=True)
    with pytest.raises(ValueError):
        atm.phase_for(wl)
    e = np.exp(1j * 0.2 * rng.standard_normal(grid.size))
    out = atm.forward(hg.Wavefront(hg.Field(e, grid), wl)).electric_field.numpy()
    back = atm.backward(hg.Wavefront(hg.Field(out, grid), wl)).electric_field.numpy()
    og = ogrids.make_pupil_grid(64, 1.0)
    internal = ogrids.make_fft_grid(og, 2, 1)

    def fresnel(x, d, adjoint=False):
        assert not ofourier.fresnel_uses_impulse_branch(og, wl, d)
        return ofourier.FourierFilterPlan(og, ofourier.fresnel_transfer_function(internal, wl, d), q=2).apply(
            x, adjoint=adjoint)

    ref = e * np.exp(1j * screens[0] / wl)
    ref = fresnel(ref, 3000.0) * np.exp(1j * screens[2] / wl)
    ref = fresnel(ref, 2000.0) * np.exp(1j * screens[1] / wl)
    assert rel_err(out, ref) < 1e-8
    rb = out * np.exp(-1j * screens[1] / wl)
    rb = fresnel(rb, 2000.0, adjoint=True) * np.exp(-1j * screens[2] / wl)
    rb = fresnel(rb, 3000.0, adjoint=True) * np.exp(-1j * screens[0] / wl)
    assert rel_err(back, rb) < 1e-8
    atm.scintillation = False
    assert rel_err(atm.forward(hg.Wavefront(hg.Field(e, grid), wl)).electric_field.numpy(),
                   e * np.exp(1j * sum(screens) / wl)) < 1e-12


def test_spectral_noise_matches_reference():
    """Multi-scale spectral noise (hcipy/util/spectral_noise.py:203-320) on the device, float64: the reference's
    seeded realization on a rectangular grid and its shifted evaluation, within 1e-10."""
    g = load_golden('spectral_noise')
    grid = _grid(g, 'grid')
    psd = hg.power_spectral_density_von_karman(float(g['r0']), float(g['L0']))
    factory = hg.SpectralNoiseFactoryMultiscale(psd, grid, int(g['oversampling']))
    noise = factory.make_random(int(g['seed']))
    screen = noise().numpy()
    assert screen.dtype == np.float64
    assert rel_err(screen, g['screen']) < 1e-10
    assert rel_err(noise.shifted(g['shift'])().numpy(), g['shifted']) < 1e-10
    assert rel_err(noise().numpy(), g['screen']) < 1e-10  # shifted() leaves the realization itself alone


def test_seeded_layer_starts_from_the_reference_screen_and_stream():
    """A layer seeded like the reference's starts from the reference's initial screen (1e-10), and its own
    generator then yields the reference's extrusion noise, so with the reference's A/B matrices the layer
    evolves into the reference's screens without any injected noise (1e-10)."""
    import copy
    g = load_golden('atmosphere')
    grid = _grid(g, 'pupil')
    layer = hg.InfiniteAtmosphericLayer(grid, float(g['cn2']), L0=25, velocity=tuple(g['velocity']),
                                        use_interpolation=True, seed=5)
    assert rel_err(layer.achromatic_screen.numpy(), g['screen0']) < 1e-10
    draw = copy.deepcopy(layer.rng).normal(0, np.sqrt(float(g['cn2'])), size=g['noise_0'].shape[1])
    assert np.array_equal(draw, g['noise_0'][0])
    _use_reference_matrices(layer, g)
    t = 0.0
    for i in range(3):
        t += float(g['dt_%d' % i])
        layer.t = t
        assert rel_err(layer.achromatic_screen.numpy(), g['screen_%d' % i]) < 1e-10, i
        assert rel_err(layer.phase_for(1.0).numpy(), g['shifted_%d' % i]) < 1e-10, i
    layer.reset()
    assert rel_err(layer.achromatic_screen.numpy(), g['screen0']) < 1e-10


@pytest.mark.parametrize('dtype', [torch.float64, torch.float32])
def test_multilayer_batched_frames_equal_layer_by_layer(dtype):
    """MultiLayerAtmosphere.evolve_until runs a frame as one extrusion launch per step index over all layers and
    one shift-and-sum pass; the same layers evolved one by one (one extrusion launch per step, one shift each,
    then the summed screen) must give the same screens and the same sum bit for bit, with layers that move 0, 1
    or several pixels a frame, in all four directions, past the ends of the ring."""
    grid = hg.make_pupil_grid(40, 2.0)
    winds = ((10.0, 0.0), (-7.5, 13.0), (0.0, 0.0), (-31.0, -22.0))

    def make():
        return [hg.InfiniteAtmosphericLayer(grid, hg.Cn_squared_from_fried_parameter(0.15, 500e-9), L0=20,
                                            velocity=v, seed=11 + i, dtype=dtype) for i, v in enumerate(winds)]
    batched, single = make(), make()
    atm = hg.MultiLayerAtmosphere(batched)
    launches = []
    t = 0.0
    for frame in range(40):
        t += 0.011
        before = hg.launch_count()
        atm.evolve_until(t)
        mid = hg.launch_count()
        for layer in single:
            layer.evolve_until(t)
        launches.append((mid - before, hg.launch_count() - mid))
        for a, b in zip(batched, single):
            assert a._row0 == b._row0 and a._col0 == b._col0
            assert torch.equal(a._shifted, b._shifted), frame
        expect = single[0]._shifted + single[1]._shifted + single[2]._shifted + single[3]._shifted
        assert torch.equal(atm.combined_screen().reshape(expect.shape), expect), frame
    # one launch per step of the fastest layer and one shift pass, against one launch per step and per layer
    assert sum(b for b, _ in launches) < 0.7 * sum(s for _, s in launches), launches
    assert all(np.array_equal(a.achromatic_screen.numpy(), b.achromatic_screen.numpy())
               for a, b in zip(batched, single))


def test_extrude_layers_rejects_a_ring_twice():
    from hcipy_gb300 import _lib
    grid = hg.make_pupil_grid(16, 1.0)
    layer = hg.InfiniteAtmosphericLayer(grid, 1e-14, L0=20, seed=3)
    noise = torch.zeros(64, dtype=torch.float64, device='cuda')
    e = layer._extrusion('right', noise)
    steps = (_lib.Extrusion * 2)(e, e)
    rc = _lib.lib().hx_atmosphere_extrude_layers(steps, 2, _lib.HX_F64, _lib.stream_handle())
    assert rc == _lib.HX_ERR_INVALID and b'twice' in _lib.lib().hx_last_error()
    assert _lib.lib().hx_atmosphere_extrude_layers(steps, 0, _lib.HX_F64, _lib.stream_handle()) == _lib.HX_OK
