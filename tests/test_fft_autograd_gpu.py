"""Adjoints of the FFT-family operators and gradients through the FFT-based propagators, on the GPU.

The padded FFT's adjoint is checked with the dot-product identity <A x, y> = <x, A^H y> (complex128, 1e-12 of
|x||A^H y|); gradients through the Fraunhofer propagator (when the planner picks an FFT), the angular-spectrum
and the Fresnel propagators are checked against the float64 oracle's adjoint (1e-10 relative), and against a
central difference of the loss (1e-6).
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import fourier as ofourier
from oracle import grids as ogrids

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def _rand(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


@pytest.mark.parametrize('q,fov,shift', [(2, 1, 0), (3, 0.5, 0), (2, 0.75, 0.3)])
def test_fft_adjoint_dot_product(q, fov, shift):
    pupil = hg.make_pupil_grid(48, 1.0)
    fft = hg.FastFourierTransform(pupil, q=q, fov=fov, shift=shift)
    rng = np.random.default_rng(3)
    x = torch.from_numpy(_rand(rng, pupil.size)).cuda()
    y = torch.from_numpy(_rand(rng, fft.output_grid.size)).cuda()
    ax = fft.forward(x).data
    ahy = fft.adjoint(y).data
    lhs = torch.vdot(y, ax).item()
    rhs = torch.vdot(ahy, x).item()
    assert abs(lhs - rhs) < 1e-12 * torch.linalg.norm(x).item() * torch.linalg.norm(ahy).item()


def test_gradient_through_fft_based_fraunhofer():
    """An integer q focal grid makes the planner pick the FFT; the loss sum |E_focal|^2 w over a region then
    differentiates through its adjoint (and through the backward propagation's adjoint)."""
    pupil = hg.make_pupil_grid(64, 1.0)
    focal = hg.make_focal_grid(2, 32)  # 128^2 at q = 2: the planner's choice is the FFT
    prop = hg.FraunhoferPropagator(pupil, focal)
    rng = np.random.default_rng(5)
    e0 = np.exp(0.3j * rng.standard_normal(pupil.size)) * (np.hypot(*pupil.points_list()) <= 0.5)
    x = torch.from_numpy(e0).cuda().requires_grad_(True)
    wts = torch.from_numpy(rng.random(focal.size)).cuda()
    out = prop.forward(hg.Wavefront(hg.Field(x, pupil), 1.0)).electric_field.data
    assert isinstance(prop.get_instance_data(pupil, focal, 1.0).fourier_transform, hg.FastFourierTransform)
    loss = ((out.real**2 + out.imag**2) * wts).sum()
    loss.backward()
    # oracle: dL/dconj(x) = A^H (2 w A x) for A = norm * FFT
    norm = 1 / (1j * 1.0 * 1.0)
    plan = ofourier.FFTPlan(ogrids.RegularGrid(pupil.delta, pupil.dims, pupil.zero), 2, 1)
    f = plan.forward(e0) * norm
    g = 2 * wts.cpu().numpy() * f
    # adjoint of the oracle FFT by the dot-product transpose: conj(norm) * scale^2 N * backward
    n_int = np.prod(plan.internal_shape)
    scale = np.prod(pupil.delta)
    ref = np.conj(norm) * plan.backward(g) * scale**2 * n_int
    assert rel_err(x.grad.cpu().numpy(), ref) < 1e-10
    # central difference along a random direction
    d = _rand(rng, pupil.size) * 1e-6

    def loss_at(e):
        o = prop.forward(hg.Wavefront(hg.Field(torch.from_numpy(e).cuda(), pupil), 1.0)).electric_field.data
        return ((o.real**2 + o.imag**2) * wts).sum().item()

    fd = (loss_at(e0 + d) - loss_at(e0 - d)) / 2
    lin = np.real(np.vdot(ref, d))  # dL = Re <grad, d>
    assert abs(fd - lin) < 1e-6 * abs(lin)
    # backward propagation (the inverse FFT) is differentiable too: its adjoint is forward / (scale^2 N conj(norm))
    y = torch.from_numpy(_rand(rng, focal.size)).cuda().requires_grad_(True)
    back = prop.backward(hg.Wavefront(hg.Field(y, focal), 1.0)).electric_field.data
    w2 = torch.from_numpy(_rand(rng, pupil.size)).cuda()
    torch.real(torch.vdot(w2, back)).backward()
    lhs = torch.vdot(w2, back).item()
    rhs = torch.vdot(y.grad, y.detach()).item()
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


@pytest.mark.parametrize('kind,d', [('asp', 0.5), ('fresnel', 0.5), ('fresnel', 200.0)])
def test_gradient_through_filter_propagators(kind, d):
    pupil = hg.make_pupil_grid(48, 8.0)
    wl = 1.6e-6
    prop = hg.AngularSpectrumPropagator(pupil, d) if kind == 'asp' else hg.FresnelPropagator(pupil, d)
    rng = np.random.default_rng(7)
    e0 = _rand(rng, pupil.size)
    w = _rand(rng, pupil.size)
    x = torch.from_numpy(e0).cuda().requires_grad_(True)
    out = prop.forward(hg.Wavefront(hg.Field(x, pupil), wl)).electric_field.data
    torch.real(torch.vdot(torch.from_numpy(w).cuda(), out)).backward()
    og = ogrids.make_pupil_grid(48, 8.0)
    internal = ogrids.make_fft_grid(og, 2, 1)
    tf = ofourier.asp_transfer_function(internal, wl, d) if kind == 'asp' else \
        ofourier.fresnel_transfer_function(internal, wl, d)
    ref = ofourier.FourierFilterPlan(og, tf, q=2).apply(w, adjoint=True)
    # dRe<w, A x>/dconj(x) = A^H w / 2 + ... torch returns the conjugate Wirtinger gradient times 2: A^H w
    assert rel_err(x.grad.cpu().numpy(), ref) < 1e-8


def test_zoom_fft_adjoint_and_fraunhofer_gradient():
    """The zoom FFT's adjoint (dot-product identity), and a Fraunhofer propagator planned on a zoom FFT is
    differentiable in both directions."""
    pupil = hg.make_pupil_grid(96, 1.0)
    focal = hg.make_focal_grid(5.3, 3)
    zf = hg.ZoomFastFourierTransform(pupil, focal.scaled(2 * np.pi))
    rng = np.random.default_rng(11)
    x = torch.from_numpy(_rand(rng, pupil.size)).cuda()
    y = torch.from_numpy(_rand(rng, focal.size)).cuda()
    lhs = torch.vdot(y, zf.forward(x).data).item()
    ahy = zf.adjoint(y).data
    rhs = torch.vdot(ahy, x).item()
    assert abs(lhs - rhs) < 1e-11 * torch.linalg.norm(x).item() * torch.linalg.norm(ahy).item()
    prop = hg.FraunhoferPropagator(pupil, focal)
    inst = prop.get_instance_data(pupil, focal, 1.0)
    if not isinstance(inst.fourier_transform, hg.ZoomFastFourierTransform):
        inst.fourier_transform = zf  # the planner's choice depends on its cost model; test the zoom path itself
    xg = x.clone().requires_grad_(True)
    out = prop.forward(hg.Wavefront(hg.Field(xg, pupil), 1.0)).electric_field.data
    torch.real(torch.vdot(y, out)).backward()
    assert abs(torch.vdot(y, out).item() - torch.vdot(xg.grad, x).item()) < 1e-10 * abs(torch.vdot(y, out).item())
    yg = y.clone().requires_grad_(True)
    back = prop.backward(hg.Wavefront(hg.Field(yg, focal), 1.0)).electric_field.data
    torch.real(torch.vdot(x, back)).backward()
    assert abs(torch.vdot(x, back).item() - torch.vdot(yg.grad, y).item()) < 1e-10 * abs(torch.vdot(x, back).item())
