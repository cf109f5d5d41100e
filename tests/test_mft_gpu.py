"""Parity of the device MFT, Fraunhofer propagator and Lyot chain with the oracle and the reference's golden vectors.

Tolerances (relative L2 error of the whole field):
  complex128 (FP64 GEMM on the device)      : 1e-12 against float64
  complex64  (FP32 CUDA-core GEMM)          : 3e-6 against float64; the reference's own
                                              complex64 result sits at ~1e-7..1e-6.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, grid_from, rel_err
from oracle import fourier as ofourier, optics as ooptics

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')

TOL64 = 1e-12
TOL32 = 3e-6


def _grids(g):
    pupil = hg.CartesianGrid(hg.SeparatedCoords([g['in_x'], g['in_y']]))
    focal = hg.CartesianGrid(hg.SeparatedCoords([g['out_x'], g['out_y']]))
    # The golden grids are regular: rebuild them as regular grids so the scalar-weight path is used.
    pupil = hg.CartesianGrid(hg.RegularCoords(g['ingrid_delta'], g['ingrid_dims'], g['ingrid_zero']))
    focal = hg.CartesianGrid(hg.RegularCoords(g['outgrid_delta'], g['outgrid_dims'], g['outgrid_zero']))
    return pupil, focal


@pytest.mark.parametrize('case', ['mft_0', 'mft_1', 'mft_2'])
@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_mft_matches_reference(case, dtype):
    g = load_golden(case)
    pupil, focal = _grids(g)
    mft = hg.MatrixFourierTransform(pupil, focal)
    e = torch.from_numpy(g['E'].astype(dtype)).cuda()
    f = torch.from_numpy(g['F'].astype(dtype)).cuda()
    fwd = mft.forward(e)
    bwd = mft.backward(f)
    assert fwd.dtype == getattr(torch, dtype)
    tol = TOL64 if dtype == 'complex128' else TOL32
    assert rel_err(fwd.numpy(), g['fwd_c128']) < tol
    assert rel_err(bwd.numpy(), g['bwd_c128']) < tol
    if dtype == 'complex64':
        # Same arithmetic class as the reference's own cgemm path.
        assert rel_err(fwd.numpy(), g['fwd_c64']) < TOL32


def test_mft_1d():
    g = load_golden('mft_1d')
    gi = hg.CartesianGrid(hg.RegularCoords(g['in_x'][1] - g['in_x'][0], len(g['in_x']), g['in_x'][0]))
    go = hg.CartesianGrid(hg.RegularCoords(g['out_x'][1] - g['out_x'][0], len(g['out_x']), g['out_x'][0]))
    mft = hg.MatrixFourierTransform(gi, go)
    assert rel_err(mft.forward(g['E']).numpy(), g['fwd_c128']) < 1e-11
    assert rel_err(mft.backward(g['F']).numpy(), g['bwd_c128']) < 1e-11


def test_mft_nonuniform_separated_weights():
    rng = np.random.default_rng(5)
    x = np.sort(rng.uniform(-0.5, 0.5, 23))
    y = np.sort(rng.uniform(-0.5, 0.5, 19))
    u = np.linspace(-20, 20, 17)
    v = np.linspace(-15, 18, 21)
    gi = hg.CartesianGrid(hg.SeparatedCoords([x, y]))
    go = hg.CartesianGrid(hg.SeparatedCoords([u, v]))
    e = rng.standard_normal(gi.size) + 1j * rng.standard_normal(gi.size)
    f = rng.standard_normal(go.size) + 1j * rng.standard_normal(go.size)
    mft = hg.MatrixFourierTransform(gi, go)
    assert rel_err(mft.forward(e).numpy(), ofourier.mft_forward(e, x, y, u, v, gi.weights)) < 1e-12
    assert rel_err(mft.backward(f).numpy(), ofourier.mft_backward(f, x, y, u, v, go.weights)) < 1e-12


@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_mft_tensor_field_batches(dtype):
    g = load_golden('mft_1')
    pupil, focal = _grids(g)
    mft = hg.MatrixFourierTransform(pupil, focal)
    rng = np.random.default_rng(1)
    e = (rng.standard_normal((3, 2, pupil.size)) + 1j * rng.standard_normal((3, 2, pupil.size))).astype(dtype)
    res = mft.forward(e).numpy()
    assert res.shape == (3, 2, focal.size)
    tol = TOL64 if dtype == 'complex128' else TOL32
    for i in range(3):
        for j in range(2):
            ref = ofourier.mft_forward(e[i, j].astype(np.complex128), g['in_x'], g['in_y'], g['out_x'], g['out_y'],
                                       pupil.weights)
            assert rel_err(res[i, j], ref) < tol
    back = mft.backward(res).numpy()
    assert back.shape == (3, 2, pupil.size)


@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_adjoint_dot_product(dtype):
    g = load_golden('mft_2')
    pupil, focal = _grids(g)
    mft = hg.MatrixFourierTransform(pupil, focal)
    rng = np.random.default_rng(2)
    x = (rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)).astype(dtype)
    y = (rng.standard_normal(focal.size) + 1j * rng.standard_normal(focal.size)).astype(dtype)
    ax = mft.forward(x).numpy().astype(np.complex128)
    ahy = mft.adjoint(y).numpy().astype(np.complex128)
    lhs = np.vdot(y, ax)
    rhs = np.vdot(ahy, x)
    tol = 1e-12 if dtype == 'complex128' else 1e-5
    assert abs(lhs - rhs) / abs(lhs) < tol


@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_fraunhofer_cfg1(dtype):
    g = load_golden('fraunhofer_cfg1')
    pupil = hg.make_pupil_grid(256, 1)
    focal = hg.make_focal_grid(q=4, num_airy=16)
    prop = hg.FraunhoferPropagator(pupil, focal)
    wf = hg.Wavefront(hg.Field(g['E'].astype(dtype), pupil), 1)
    out = prop.forward(wf).electric_field
    assert out.grid is focal
    tol = TOL64 if dtype == 'complex128' else TOL32
    assert rel_err(out.numpy(), g['focal_c128']) < tol
    back = prop.backward(hg.Wavefront(hg.Field(g['focal_c128'].astype(dtype), focal), 1)).electric_field
    assert rel_err(back.numpy(), g['back_c128']) < tol
    if dtype == 'complex64':
        # Intensity error normalised to the peak, the contrast-style figure.
        ni_err = np.abs(np.abs(out.numpy())**2 - np.abs(g['focal_c128'])**2).max() / np.abs(g['focal_c128']).max()**2
        assert ni_err < 1e-6


@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_lyot_chain_matches_reference(dtype):
    g = load_golden('lyot')
    pupil = hg.make_pupil_grid(128, 1)
    fpm_grid = hg.make_focal_grid(8, 8)
    focal = hg.make_focal_grid(4, 16)
    fpm = hg.Field(g['fpm'], fpm_grid)
    stop = hg.Field(g['stop'], pupil)
    lyot = hg.LyotCoronagraph(pupil, fpm, stop)
    prop = hg.FraunhoferPropagator(pupil, focal)
    wf = hg.Wavefront(hg.Field(g['E'].astype(dtype), pupil), 1)
    lp = lyot.forward(wf)
    tol = TOL64 if dtype == 'complex128' else 2e-5
    assert rel_err(lp.electric_field.numpy(), g['lyot_c128']) < tol
    img = prop.forward(lp).electric_field.numpy()
    # Normalised intensity error against the reference float64 chain.
    ni = np.abs(img)**2 * focal.weights / g['ref_peak']
    ni_ref = np.abs(g['image_c128'])**2 * focal.weights / g['ref_peak']
    assert np.abs(ni - ni_ref).max() < (1e-13 if dtype == 'complex128' else 2e-9)


def test_lyot_unfused_path_agrees():
    g = load_golden('lyot')
    pupil = hg.make_pupil_grid(128, 1)
    fpm_grid = hg.make_focal_grid(8, 8)
    fpm = hg.Apodizer(hg.Field(g['fpm'], fpm_grid))
    lyot = hg.LyotCoronagraph(pupil, fpm, hg.Field(g['stop'], pupil), focal_plane_mask_grid=fpm_grid)
    out = lyot.forward(hg.Wavefront(hg.Field(g['E'], pupil), 1)).electric_field.numpy()
    assert rel_err(out, g['lyot_c128']) < TOL64


def test_errors_and_fault_injection(monkeypatch):
    pupil = hg.make_pupil_grid(16, 1)
    with pytest.raises(ValueError):
        hg.MatrixFourierTransform(pupil, hg.make_uniform_grid(7, 1.0))
    mft = hg.MatrixFourierTransform(pupil, hg.make_focal_grid(2, 4))
    with pytest.raises(ValueError):
        mft.forward(torch.zeros(15, dtype=torch.complex64, device='cuda'))
    monkeypatch.setenv('HX_FAULT', 'plan')
    with pytest.raises(hg.HXError) as ei:
        hg.MatrixFourierTransform(pupil, hg.make_focal_grid(2, 3)).forward(torch.zeros(256, device='cuda'))
    assert ei.value.code == -6
    monkeypatch.setenv('HX_FAULT', 'launch')
    with pytest.raises(hg.HXError):
        mft.forward(torch.zeros(256, dtype=torch.complex64, device='cuda'))
    monkeypatch.delenv('HX_FAULT')
    # make_focal_grid(2, 4) is 16 x 16.
    assert mft.forward(torch.ones(256, dtype=torch.complex64, device='cuda')).shape == (256,)


def test_inputs_are_not_modified():
    g = load_golden('lyot')
    pupil = hg.make_pupil_grid(128, 1)
    fpm_grid = hg.make_focal_grid(8, 8)
    lyot = hg.LyotCoronagraph(pupil, hg.Field(g['fpm'], fpm_grid), hg.Field(g['stop'], pupil))
    e = torch.from_numpy(g['E']).cuda()
    keep = e.clone()
    lyot.forward(hg.Wavefront(hg.Field(e, pupil), 1))
    assert torch.equal(e, keep)


def test_native_kernels_launch():
    before = hg.launch_count()
    mft = hg.MatrixFourierTransform(hg.make_pupil_grid(32), hg.make_focal_grid(2, 4))
    mft.forward(torch.ones(1024, dtype=torch.complex64, device='cuda'))
    torch.cuda.synchronize()
    assert hg.launch_count() - before >= 2
