"""The split-operand tcgen05 MFT (precision='split') against the float64 oracle and its arithmetic model.

The split form cuts every operand into fixed-point slices (6, 11, 11 bits) and
sums the kept slice products exactly, so its error does not grow with the
transform length as FP32 accumulation does.  Tolerances:
  device result vs the numpy model of the split arithmetic : 2e-8 relative (same slices of the inputs; the device
                                                             slices the float-float intermediate in FP32, which
                                                             can move the last slice of an element by one unit;
                                                             a wrong level or scale shows at 1e-4 or worse)
  MFT fields (complex128 results), relative L2 vs float64  : 2e-8 (~2^-29 per operand element)
  Lyot dark hole (3-15 lambda/D), 512^2 pupil              : max |NI - NI_fp64| < 5e-12 and < 1/20 of FP32's
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, rel_err
import split_model
from oracle import fourier as ofourier, optics as ooptics
from oracle.grids import RegularGrid

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def regular(g, prefix):
    return hg.CartesianGrid(hg.RegularCoords(g[prefix + '_delta'], g[prefix + '_dims'], g[prefix + '_zero']))


def og(grid):
    return RegularGrid(grid.delta, grid.dims, grid.zero)


def test_split_mft_forward_small():
    g = load_golden('mft_0')
    pupil, focal = regular(g, 'ingrid'), regular(g, 'outgrid')
    e = torch.from_numpy(g['E'].astype(np.complex64)).cuda()
    split = hg.MatrixFourierTransform(pupil, focal, precision='split')
    out = split.forward(e).numpy()
    ref = ofourier.mft_forward(e.cpu().numpy().astype(complex), g['in_x'], g['in_y'], g['out_x'], g['out_y'],
                               pupil.weights)
    assert split._plan(torch.complex64).status() == 0
    model = split_model.mft_forward(e.cpu().numpy(), g['in_x'], g['in_y'], g['out_x'], g['out_y'], pupil.weights)
    assert out.dtype == np.complex128
    assert rel_err(out, model) < 2e-8
    assert rel_err(out, ref) < 2e-8


@pytest.mark.parametrize('case', ['mft_0', 'mft_1', 'mft_2'])
def test_split_mft_all_directions(case):
    g = load_golden(case)
    pupil, focal = regular(g, 'ingrid'), regular(g, 'outgrid')
    x, y, u, v = g['in_x'], g['in_y'], g['out_x'], g['out_y']
    e = g['E'].astype(np.complex64)
    f = g['F'].astype(np.complex64)
    split = hg.MatrixFourierTransform(pupil, focal, precision='split')
    plain = hg.MatrixFourierTransform(pupil, focal)
    checks = [
        (split.forward(e), plain.forward(e), ofourier.mft_forward(e.astype(complex), x, y, u, v, pupil.weights)),
        (split.backward(f), plain.backward(f), ofourier.mft_backward(f.astype(complex), x, y, u, v, focal.weights)),
        (split.adjoint(f), plain.adjoint(f), ofourier.mft_adjoint(f.astype(complex), x, y, u, v, pupil.weights)),
    ]
    for got, fp32, ref in checks:
        assert rel_err(got.numpy(), ref) < 2e-8
    assert split._plan(torch.complex64).status() == 0


def test_split_mft_batched_and_nonuniform():
    rng = np.random.default_rng(3)
    xg = np.sort(rng.uniform(-0.5, 0.5, 70))
    yg = np.sort(rng.uniform(-0.5, 0.5, 66))
    ug = np.linspace(-30, 30, 90)
    vg = np.linspace(-25, 28, 71)
    gi = hg.CartesianGrid(hg.SeparatedCoords([xg, yg]))
    go = hg.CartesianGrid(hg.SeparatedCoords([ug, vg]))
    split = hg.MatrixFourierTransform(gi, go, precision='split')
    e = (rng.standard_normal((2, 3, gi.size)) + 1j * rng.standard_normal((2, 3, gi.size))).astype(np.complex64)
    out = split.forward(e).numpy()
    for i in range(2):
        for j in range(3):
            ref = ofourier.mft_forward(e[i, j].astype(complex), xg, yg, ug, vg, gi.weights)
            assert rel_err(out[i, j], ref) < 2e-8
    f = (rng.standard_normal((4, go.size)) + 1j * rng.standard_normal((4, go.size))).astype(np.complex64)
    back = split.backward(f).numpy()
    for i in range(4):
        ref = ofourier.mft_backward(f[i].astype(complex), xg, yg, ug, vg, go.weights)
        assert rel_err(back[i], ref) < 2e-8
    assert split._plan(torch.complex64).status() == 0


def _lyot_ni_errors(n):
    from hcipy_gb300 import workloads
    w = workloads.lyot_workload(pupil_n=n)
    pupil, fpm_grid, focal = w['pupil'], w['fpm_grid'], w['focal']
    chain64 = ooptics.LyotChain(og(pupil), og(fpm_grid), og(focal), w['fpm'], w['stop'])
    ref = chain64(w['E'])
    peak = np.abs(chain64.image(w['aperture'].astype(complex))).max()**2
    mask = workloads.dark_hole_mask(focal)
    errs = {}
    for precision in ('fp32', 'split'):
        lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], fpm_grid), hg.Field(w['stop'], pupil),
                                  precision=precision)
        prop = hg.FraunhoferPropagator(pupil, focal, precision=precision)
        img = prop(lyot(hg.Wavefront(hg.Field(w['E'].astype(np.complex64), pupil), 1.0))).electric_field.numpy()
        d = np.abs(np.abs(img.astype(complex))**2 - np.abs(ref)**2)[mask] / peak
        errs[precision] = (d.max(), d.mean())
    return errs


def test_split_lyot_dark_hole_512():
    errs = _lyot_ni_errors(512)
    assert errs['split'][0] < 5e-12, errs
    assert errs['split'][0] < errs['fp32'][0] / 20, errs


@pytest.mark.parametrize('tile', ['64,1', '128,1', '64,3', '128,4', '112,1', '112,2'])
def test_split_tile_configurations(tile):
    """Both tile widths, with and without split K, against float64 (the heuristic picks one per GEMM)."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    env = dict(os.environ, HX_SPLIT_TILE=tile)
    res = subprocess.run([sys.executable, os.path.join(here, 'split_tile_case.py')], env=env,
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    fields = res.stdout.split()
    errs = [float(x) for x in fields[:-1]]
    assert int(fields[-1]) == 0
    assert len(errs) == 6 and max(errs) < 2e-8, errs


def test_split_complex128_wide_range():
    """complex128 fields from 1e-20 to 1e20 (the float64 <-> float-float conversions), each against float64."""
    rng = np.random.default_rng(5)
    n_in, n_out = 96, 80
    xg = (np.arange(n_in) - n_in / 2 + 0.5) / n_in
    ug = (np.arange(n_out) - n_out / 2 + 0.5) * 0.41
    gi = hg.CartesianGrid(hg.RegularCoords(1.0 / n_in, [n_in, n_in], [xg[0], xg[0]]))
    go = hg.CartesianGrid(hg.RegularCoords(0.41, [n_out, n_out], [ug[0], ug[0]]))
    split = hg.MatrixFourierTransform(gi, go, precision='split')
    scales = np.array([1e-20, 3e-7, 1.0, 7e8, 1e20])
    base = rng.standard_normal((len(scales), gi.size)) + 1j * rng.standard_normal((len(scales), gi.size))
    e = base * scales[:, None]
    out = split.forward(torch.from_numpy(e).cuda()).numpy()
    assert out.dtype == np.complex128
    for i in range(len(scales)):
        ref = ofourier.mft_forward(e[i], xg, xg, ug, ug, gi.weights)
        assert rel_err(out[i], ref) < 2e-8, (scales[i], rel_err(out[i], ref))
    assert split._plan(torch.complex64).status() == 0


def test_split_throughput_schedule_all_directions():
    """The throughput tile policy (no K split, least padded tile) on a shape that the latency policy splits:
    forward, backward and adjoint against float64, and switching the schedule of an existing plan."""
    pupil = hg.make_pupil_grid(256, 1.0)
    focal = hg.make_focal_grid(3.7, 19)  # 140^2: the throughput policy takes 112-column tiles
    rng = np.random.default_rng(8)
    e = (rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)).astype(np.complex64)
    f = (rng.standard_normal(focal.size) + 1j * rng.standard_normal(focal.size)).astype(np.complex64)
    x, y = pupil.separated_coords
    u, v = focal.separated_coords
    ref_f = ofourier.mft_forward(e.astype(complex), x, y, u, v, pupil.weights)
    ref_b = ofourier.mft_backward(f.astype(complex), x, y, u, v, focal.weights)
    ref_a = ofourier.mft_adjoint(f.astype(complex), x, y, u, v, pupil.weights)
    mft = hg.MatrixFourierTransform(pupil, focal, precision='split', schedule='throughput')
    et, ft = torch.from_numpy(e).cuda(), torch.from_numpy(f).cuda()
    assert rel_err(mft.forward(et).numpy(), ref_f) < 2e-8
    assert rel_err(mft.backward(ft).numpy(), ref_b) < 2e-8
    assert rel_err(mft.adjoint(ft).numpy(), ref_a) < 2e-8
    mft.schedule = 'latency'
    assert rel_err(mft.forward(et).numpy(), ref_f) < 2e-8
    assert mft._plan(torch.complex64).status() == 0
    with pytest.raises(ValueError):
        mft.schedule = 'fastest'


def test_split_beyond_one_cta_exact_range():
    """A CTA's level-0 sum is exact up to K' = 4096, so a 2080-point axis (K' = 4160) is always split across
    CTAs (float-float partials): forward and backward against the float64 oracle at the split tolerance.  Grids
    beyond 8192 points per axis are refused loudly (HX_ERR_UNSUPPORTED) before anything is allocated."""
    pupil = hg.make_pupil_grid(2080, 1)
    focal = hg.make_focal_grid(2, 6)
    uv = focal.scaled(2 * np.pi)
    mft = hg.MatrixFourierTransform(pupil, uv, precision='split')
    rng = np.random.default_rng(12)
    e = (rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)).astype(np.complex64)
    x, y = pupil.separated_coords
    u, v = uv.separated_coords
    w_in = float(np.asarray(pupil.weights).ravel()[0])
    fwd = mft.forward(hg.Field(torch.from_numpy(e).cuda(), pupil)).data.cpu().numpy()
    ref = ofourier.mft_forward(e.astype(np.complex128), x, y, u, v, w_in)
    assert rel_err(fwd, ref) < 2e-8, rel_err(fwd, ref)
    f = (rng.standard_normal(uv.size) + 1j * rng.standard_normal(uv.size)).astype(np.complex64)
    w_out = float(np.asarray(uv.weights).ravel()[0])
    back = mft.backward(hg.Field(torch.from_numpy(f).cuda(), uv)).data.cpu().numpy()
    ref_b = ofourier.mft_backward(f.astype(np.complex128), x, y, u, v, w_out)
    assert rel_err(back, ref_b) < 2e-8, rel_err(back, ref_b)
    big = hg.make_pupil_grid(8200, 1)
    mft_big = hg.MatrixFourierTransform(big, uv, precision='split')
    with pytest.raises(hg.HXError, match='at most 8192 points per axis'):
        mft_big.forward(hg.Field(torch.ones(big.size, dtype=torch.complex64, device='cuda'), big))


@pytest.mark.parametrize('n,dtype', [(128, np.complex64), (384, np.complex128), (2304, np.complex64)])
def test_lyot_execute_with_the_image_plan(n, dtype):
    """hx_lyot_execute given the image transform's plan (coronagraph and lens in one call, the Lyot plane sliced
    for the image transform by the Babinet row pass itself, never stored) against LyotCoronagraph followed by
    FraunhoferPropagator (two calls), split precision, batch 2: the same image within 1e-12, and within 2e-8 of the
    float64 oracle chain.  Pupils of 128, 384 and 2304 points per row: one, one and three row groups of 1024
    points per thread block."""
    from hcipy_gb300 import _lib
    from oracle.grids import RegularGrid as OG
    rng = np.random.default_rng(n)
    pupil = hg.make_pupil_grid(n, 1)
    fpm_grid = hg.make_focal_grid(4, 6)
    focal = hg.make_focal_grid(3, 10)
    r = np.hypot(fpm_grid.x, fpm_grid.y)
    fpm = (r > 2.5).astype(float) + 0.0j
    stop = (np.hypot(pupil.x, pupil.y) < 0.45).astype(float) + 0.0j
    lyot = hg.LyotCoronagraph(pupil, hg.Field(fpm, fpm_grid), hg.Field(stop, pupil), precision='split')
    prop = hg.FraunhoferPropagator(pupil, focal, precision='split')
    ap = (np.hypot(pupil.x, pupil.y) < 0.5).astype(float)
    e = (ap[None, :] * np.exp(1j * 0.05 * rng.standard_normal((2, pupil.size)))).astype(dtype)
    t = torch.from_numpy(e).cuda()
    two = prop.forward(lyot.forward(hg.Wavefront(hg.Field(t, pupil), 1.0))).electric_field.data
    inst = lyot.prop.get_instance_data(pupil, None, 1.0)
    ft = inst.fourier_transform
    one_minus, stop_t = lyot._fused_masks(t.dtype)
    a_fwd = complex(ft._w_in_scalar) * inst.norm_factor
    a_bwd = complex(ft._w_out_scalar / (2 * np.pi)**ft.ndim) / inst.norm_factor
    pinst = prop.get_instance_data(pupil, None, 1.0)
    pft = pinst.fourier_transform
    a_img = complex(pft._w_in_scalar) * pinst.norm_factor
    out = torch.empty((2, focal.size), dtype=torch.complex128, device='cuda')
    lib = _lib.lib()
    plan, img_plan = ft._plan(t.dtype), pft._plan(t.dtype)
    nbytes = int(lib.hx_lyot_workspace_bytes(plan.handle, img_plan.handle, 2))
    ws = _lib.workspace(nbytes, t.device)
    rc = lib.hx_lyot_execute(plan.handle, img_plan.handle, 2, _lib.dptr(t), _lib.dtype_code(t.dtype),
                             _lib.dptr(one_minus), _lib.dptr(stop_t), a_fwd.real, a_fwd.imag, a_bwd.real, a_bwd.imag,
                             a_img.real, a_img.imag, None, _lib.HX_C128, _lib.dptr(out), _lib.HX_C128, _lib.dptr(ws),
                             nbytes, _lib.stream_handle())
    _lib.check(rc, 'hx_lyot_execute')
    one = out.cpu().numpy()
    assert rel_err(one, two.cpu().numpy()) < 1e-12
    og = lambda g: OG(g.delta, g.dims, g.zero)  # noqa: E731
    chain = ooptics.LyotChain(og(pupil), og(fpm_grid), og(focal), fpm.real, stop.real)
    for b in range(2):
        assert rel_err(one[b], chain(e[b].astype(complex))) < 2e-8
