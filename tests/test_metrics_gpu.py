"""Dark-hole contrast sums on the device (hcipy_gb300.intensity_sum): compensated float-float reductions against
float64 numpy, determinism, the gradient 2 w E, and the DM-gradient loss built on them.

Tolerances: the products |E|^2 of complex64 values are exact in float-float and the sums compensated, so both
complex64 and complex128 fields agree with float64 numpy to 1e-13 relative; gradients to 1e-12."""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


@pytest.mark.parametrize('dtype', [torch.complex64, torch.complex128])
@pytest.mark.parametrize('shape', [(), (3,), (2, 3)])
def test_intensity_sums_match_float64(dtype, shape):
    rng = np.random.default_rng(30)
    n = 70001  # not a multiple of the chunk size
    e = (rng.standard_normal(shape + (n,)) + 1j * rng.standard_normal(shape + (n,))) * 1e-3
    e_t = torch.from_numpy(e).to('cuda', dtype)
    e_h = e_t.cpu().numpy().astype(np.complex128)  # the values the device sees
    w = (rng.random(n) > 0.5).astype(np.float32) * rng.random(n).astype(np.float32)
    for weights in (None, w):
        got = hg.intensity_sum(e_t, weights)
        assert got.dtype == torch.float64 and tuple(got.shape) == shape
        ref = (np.abs(e_h)**2 * (1.0 if weights is None else weights.astype(np.float64))).sum(-1)
        assert rel_err(got.cpu().numpy(), ref) < 1e-13
        assert torch.equal(got, hg.intensity_sum(e_t, weights))  # fixed reduction order


def test_intensity_sum_gradient_and_mean():
    rng = np.random.default_rng(31)
    n = 4099
    e = torch.from_numpy(rng.standard_normal((4, n)) + 1j * rng.standard_normal((4, n))).cuda().requires_grad_(True)
    w = torch.from_numpy(rng.random(n)).float().cuda()
    g = torch.from_numpy(rng.standard_normal(4)).cuda()
    (hg.intensity_sum(e, w) * g).sum().backward()
    ref = 2 * g[:, None] * w.double()[None, :] * e.detach()
    assert rel_err(e.grad.cpu().numpy(), ref.cpu().numpy()) < 1e-12
    mask = rng.random(n) > 0.7
    m = hg.mean_intensity_in_roi(e.detach()[0], mask)
    assert abs(float(m) - float((e.detach()[0].abs()**2).cpu().numpy()[mask].mean())) < 1e-13 * float(m)
    assert tuple(hg.intensity_sum(torch.empty((0, n), dtype=torch.complex64, device='cuda')).shape) == (0,)


def test_dm_gradient_with_intensity_sum():
    """The DM-gradient loss (intensity over a half annulus behind DM, Lyot and lens) from intensity_sum: the same
    loss and actuator gradient as the element-wise torch formula."""
    from hcipy_gb300 import workloads
    w = workloads.dm_gradient_workload(pupil_n=128, n_act=12, nvec=3, fpm_q=4, fpm_num_airy=12, final_q=3.3,
                                       final_num_airy=10)
    pupil = w['pupil']
    lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], w['fpm_grid']), hg.Field(w['stop'], pupil),
                              precision='split')
    prop = hg.FraunhoferPropagator(pupil, w['focal'], precision='split')
    dm = hg.DeformableMirror(w['influence'])
    e0 = torch.from_numpy(w['aperture'].astype(np.complex64)).cuda()
    roi = torch.from_numpy(w['roi'].astype(np.float32)).cuda()
    out = []
    for fused in (True, False):
        a = torch.from_numpy(w['actuators'].astype(np.float32)).cuda().requires_grad_(True)
        dm.actuators = a
        img = prop.forward(lyot.forward(dm.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0)))).electric_field.data
        loss = hg.intensity_sum(img, roi).sum() if fused else ((img.real**2 + img.imag**2) * roi).sum()
        loss.backward()
        out.append((float(loss.detach()), a.grad.cpu().numpy()))
    assert abs(out[0][0] - out[1][0]) < 1e-12 * out[1][0]
    assert rel_err(out[0][1], out[1][1]) < 1e-6
