"""Broadband imaging with uneven focal grids, CUDA-graph capture and the tile autotuner, on the GPU.

Tolerances: complex64 fields on the FP32 path 3e-6 relative to the float64 oracle; the split form 2e-8;
a graph replay reproduces the direct call exactly (the same kernels on the same data).
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import optics as ooptics
from oracle.grids import RegularGrid

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def _og(g):
    return RegularGrid(g.delta, g.dims, g.zero)


@pytest.mark.parametrize('precision,tol', [('fp32', 3e-6), ('split', 2e-8)])
def test_broadband_matches_oracle_and_graph_replay(precision, tol):
    from hcipy_gb300 import workloads
    pupil = hg.make_pupil_grid(128, 1)
    wls = np.linspace(0.9, 1.1, 5)
    grids = hg.diffraction_scaled_focal_grids(3.3, 9, wls, 1.0)  # q keeps the planner on the MFT
    assert len({int(g.dims[0]) for g in grids}) > 1
    imager = hg.BroadbandImager(pupil, wls, grids, precision=precision)
    rng = np.random.default_rng(1)
    ap = workloads.circular_aperture(pupil, 1.0)
    e = (ap * np.exp(1j * 0.3 * rng.standard_normal(pupil.size))).astype(np.complex64)
    e_t = torch.from_numpy(e).cuda()
    out = imager(e_t)
    for wl, g, img in zip(wls, grids, out):
        ref = ooptics.fraunhofer_forward(e.astype(complex), _og(pupil), _og(g), wavelength=wl)
        assert rel_err(img.cpu().numpy(), ref) < tol, (wl, rel_err(img.cpu().numpy(), ref))
    imager.capture(e_t)
    e2 = torch.from_numpy((ap * np.exp(1j * 0.3 * rng.standard_normal(pupil.size))).astype(np.complex64)).cuda()
    direct = [x.clone() for x in imager(e2)]
    replayed = imager.replay(e2)
    for a, b in zip(direct, replayed):
        assert torch.equal(a, b)


def test_graph_with_atmosphere_and_autotuner():
    """An atmospheric layer ahead of the lens inside the captured graph: evolving the layer between replays
    changes the screen the graph reads.  The split GEMMs are autotuned during the warm-up, never inside capture."""
    from hcipy_gb300 import _lib
    pupil = hg.make_pupil_grid(96, 1)
    layer = hg.InfiniteAtmosphericLayer(pupil, hg.Cn_squared_from_fried_parameter(0.3, 500e-9), L0=20,
                                        velocity=5.0, seed=2, dtype=torch.float32)
    wls = [0.95, 1.05]
    imager = hg.BroadbandImager(pupil, wls, hg.diffraction_scaled_focal_grids(3.3, 8, wls, 1.0), precision="split",
                                pre=layer.forward)
    _lib.autotune(True)
    try:
        e = torch.ones(pupil.size, dtype=torch.complex64, device='cuda')
        imager.capture(e)
        assert _lib.autotune_entries() > 0
        first = [x.clone() for x in imager.replay(e)]
        layer.evolve_until(0.05)
        second = [x.clone() for x in imager.replay(e)]
        direct = imager(e)
        for a, b in zip(second, direct):
            assert torch.equal(a, b)
        assert any(not torch.equal(a, b) for a, b in zip(first, second))
    finally:
        _lib.autotune(False)


def test_broadband_through_multilayer_atmosphere():
    """The broadband workload's form at a small size: three float32 layers ahead of uneven focal grids, the
    graph captured once and replayed per frame after the layers evolve; each replay equals the direct call and,
    at every wavelength, the float64 oracle on the field the device propagated."""
    from hcipy_gb300 import workloads
    from hcipy_gb300.kernels import apply_phase
    w = workloads.broadband_turbulence_workload(pupil_n=96, diameter=2.0, num_wavelengths=5, q=3.3, num_airy=8)
    pupil, wls, grids = w['pupil'], w['wavelengths'], w['focal_grids']
    assert len({int(g.dims[0]) for g in grids}) > 1
    layers = [hg.InfiniteAtmosphericLayer(pupil, hg.Cn_squared_from_fried_parameter(lay['r0'], 500e-9),
                                          L0=w['L0'], velocity=lay['velocity'], seed=3 + i, dtype=torch.float32)
              for i, lay in enumerate(w['layers'])]
    atm = hg.MultiLayerAtmosphere(layers)
    ap = torch.from_numpy(w['aperture'].astype(np.complex64)).cuda()
    for precision, tol in (('fp32', 3e-6), ('split', 2e-8)):
        atm.reset()
        imager = hg.BroadbandImager(pupil, wls, grids, focal_length=w['focal_length'], precision=precision,
                                    pre=atm.forward).capture(ap)
        assert imager.graph_kernels >= 2 * len(wls)
        t = 0.0
        for _ in range(3):
            t += 4 * w['frame_time']
            atm.evolve_until(t)
            replayed = [x.clone() for x in imager.replay(ap)]
            direct = imager(ap)
            for a, b in zip(replayed, direct):
                assert torch.equal(a, b)
        for wl, g, img in zip(wls, grids, replayed):
            e = apply_phase(ap, atm.combined_screen(), 1.0 / wl).cpu().numpy().astype(np.complex128)
            ref = ooptics.fraunhofer_forward(e, _og(pupil), _og(g), wavelength=wl, focal_length=w['focal_length'])
            assert rel_err(img.cpu().numpy(), ref) < tol, (precision, wl, rel_err(img.cpu().numpy(), ref))


def test_captured_dm_probes():
    """A batch of DM probe commands through the DM, the Lyot coronagraph and the lens, recorded once as a CUDA
    graph (CapturedCall): replays equal the direct call for each new set of commands."""
    from hcipy_gb300 import workloads
    w = workloads.dm_gradient_workload(pupil_n=128, n_act=12, nvec=3, fpm_q=4, fpm_num_airy=12, final_q=3.3,
                                       final_num_airy=10)
    pupil = w['pupil']
    lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], w['fpm_grid']), hg.Field(w['stop'], pupil))
    prop = hg.FraunhoferPropagator(pupil, w['focal'])
    dm = hg.DeformableMirror(w['influence'])
    e0 = torch.from_numpy(w['aperture'].astype(np.complex64)).cuda()

    def measure(c):
        dm.actuators = c
        e = dm.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0))
        img = prop.forward(lyot.forward(e)).electric_field.data
        return img.real**2 + img.imag**2

    cmd = torch.from_numpy(w['actuators'].astype(np.float32)).cuda()
    graph = hg.CapturedCall(measure, cmd)
    assert graph.graph_kernels > 0
    for k in range(3):
        c = cmd * (1 + k)
        replayed = graph(c).clone()
        assert torch.equal(replayed, measure(c))
    first = graph(cmd).clone()
    assert not torch.equal(first, graph(2 * cmd))
    with pytest.raises(ValueError):
        graph(cmd, cmd)


def test_phase_screen_fused_into_the_slicing():
    """With an atmosphere without scintillation as ``pre`` (the element or its bound ``forward``), the split
    transforms apply its phase while slicing their input (``hx_mft_execute_phase``): the images equal those of the
    phase kernel followed by the transform (an opaque ``pre`` forces that path) bit for bit, directly,
    concurrently and from a captured graph that replays the current screens; complex128 fields and the FP32 form
    keep the separate phase kernel."""
    from hcipy_gb300 import _lib, workloads
    w = workloads.broadband_turbulence_workload(pupil_n=96, diameter=2.0, num_wavelengths=4, q=3.3, num_airy=8)
    pupil, wls, grids = w['pupil'], w['wavelengths'], w['focal_grids']
    layers = [hg.InfiniteAtmosphericLayer(pupil, hg.Cn_squared_from_fried_parameter(lay['r0'], 500e-9),
                                          L0=w['L0'], velocity=lay['velocity'], seed=8 + i, dtype=torch.float32)
              for i, lay in enumerate(w['layers'])]
    atm = hg.MultiLayerAtmosphere(layers)
    atm.evolve_until(4 * w['frame_time'])
    e = torch.from_numpy(w['aperture'].astype(np.complex64)).cuda()
    kw = dict(focal_length=w['focal_length'], precision='split')
    fused = hg.BroadbandImager(pupil, wls, grids, pre=atm.forward, **kw)
    by_element = hg.BroadbandImager(pupil, wls, grids, pre=atm, **kw)
    plain = hg.BroadbandImager(pupil, wls, grids, pre=lambda wf: atm.forward(wf), **kw)
    assert fused._phase_screen() is not None and by_element._phase_screen() is not None
    assert plain._phase_screen() is None
    for concurrent in (False, True):
        a = fused.forward(e, concurrent=concurrent)
        b = plain.forward(e, concurrent=concurrent)
        c = by_element.forward(e, concurrent=concurrent)
        torch.cuda.synchronize()
        for x, y, z in zip(a, b, c):
            assert torch.equal(x, y) and torch.equal(x, z)
    fused.capture(e)
    plain.capture(e)
    atm.evolve_until(8 * w['frame_time'])
    for x, y in zip(fused.replay(e), plain.replay(e)):
        assert torch.equal(x, y)
    # not fusable: complex128 fields, FP32 transforms
    prop = fused.props[0]
    assert not prop.phase_screen_fusable(e.to(torch.complex128), atm.combined_screen(), wls[0])
    fp32 = hg.FraunhoferPropagator(pupil, grids[0], focal_length=w['focal_length'])
    assert fp32.forward_phase_screen(e, atm.combined_screen(), 1 / wls[0], wls[0]) is None
    # the C ABI refuses a plain plan
    ft = fp32.get_instance_data(pupil, None, wls[0]).fourier_transform
    plan = ft._plan(torch.complex64)
    out = torch.empty(grids[0].size, dtype=torch.complex128, device='cuda')
    rc = _lib.lib().hx_mft_execute_phase(plan.handle, 1, _lib.dptr(e), _lib.dptr(atm.combined_screen()), 1.0,
                                         _lib.dptr(out), _lib.HX_C128, 1.0, 0.0, None, 0, _lib.stream_handle())
    assert rc == _lib.HX_ERR_INVALID
