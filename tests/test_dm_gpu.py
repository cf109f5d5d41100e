"""Deformable mirror, phase kernels and the adjoint (autograd) forms of the operators, on the GPU.

Tolerances:
  DM surface / reflection vs the reference (float64)      : 1e-12 relative (sparse sums in another order)
  float32 surfaces                                        : 1e-6
  adjoint dot products |<w, A x> - <A^H w, x>| / (|w| |A x|), float64 : 1e-12 (two float64 transforms)
  the same, split precision                                          : 1e-8 (~2^-29 per operand element)
  gradient vs central differences (float64 chain)         : 1e-6 relative (difference step and curvature)
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, rel_err
from oracle import optics as ooptics
from oracle.grids import RegularGrid

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def _grid(rec, prefix):
    return hg.CartesianGrid(hg.RegularCoords(rec[prefix + '_delta'], rec[prefix + '_dims'], rec[prefix + '_zero']))


def _vdot(a, b):
    return complex(torch.vdot(a.reshape(-1).to(torch.complex128), b.reshape(-1).to(torch.complex128)).item())


def test_dm_surface_and_reflection_match_reference():
    g = load_golden('dm')
    grid = _grid(g, 'pupil')
    inf = hg.make_gaussian_influence_functions(grid, 8, 1 / 8, crosstalk=0.15)
    dm = hg.DeformableMirror(inf, dtype=torch.float64)
    dm.actuators = g['actuators']
    assert rel_err(dm.surface.numpy(), g['surface']) < 1e-12
    wf = hg.Wavefront(hg.Field(g['E'], grid), 1.0)
    out = dm.forward(wf).electric_field.numpy()
    assert out.dtype == np.complex128
    assert rel_err(out, g['fwd_c128']) < 1e-12
    back = dm.backward(dm.forward(wf)).electric_field.numpy()
    assert rel_err(back, g['E']) < 1e-12
    dm32 = hg.DeformableMirror(inf)
    dm32.actuators = g['actuators']
    assert rel_err(dm32.surface.numpy(), g['surface']) < 1e-6
    assert np.allclose(dm.phase_for(0.5).numpy(), 8 * np.pi * g['surface'], rtol=1e-12, atol=0)


def test_dm_batched_surfaces_and_transpose():
    g = load_golden('dm')
    grid = _grid(g, 'pupil')
    inf = hg.make_gaussian_influence_functions(grid, 8, 1 / 8, crosstalk=0.15)
    m = inf.transformation_matrix.toarray()
    rng = np.random.default_rng(1)
    a = rng.standard_normal((5, inf.num_modes))
    basis = inf.device_basis(torch.device('cuda'), torch.float64)
    s = basis.apply(torch.from_numpy(a)).cpu().numpy()
    assert rel_err(s, a @ m.T) < 1e-12
    w = rng.standard_normal((5, grid.size))
    gt = basis.apply_transpose(torch.from_numpy(w)).cpu().numpy()
    assert rel_err(gt, w @ m) < 1e-12
    assert abs(np.sum(s * w) - np.sum(a * gt)) < 1e-10 * abs(np.sum(s * w))


def test_phase_apply_gradient_matches_finite_differences():
    from hcipy_gb300.autograd import phase_apply
    rng = np.random.default_rng(2)
    n = 300
    e = torch.from_numpy(rng.standard_normal(n) + 1j * rng.standard_normal(n)).cuda()
    s0 = rng.standard_normal((3, n))
    w = torch.from_numpy(rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))).cuda()

    def loss(s_t):
        y = phase_apply(e, s_t, 0.7)
        return (torch.abs((y * w).sum(-1))**2).sum()

    s = torch.from_numpy(s0).cuda().requires_grad_(True)
    loss(s).backward()
    grad = s.grad.cpu().numpy()
    h = 1e-6
    for (b, i) in [(0, 3), (1, 150), (2, 299)]:
        sp = s0.copy()
        sp[b, i] += h
        sm = s0.copy()
        sm[b, i] -= h
        with torch.no_grad():
            fd = (loss(torch.from_numpy(sp).cuda()) - loss(torch.from_numpy(sm).cuda())).item() / (2 * h)
        assert abs(fd - grad[b, i]) < 1e-6 * max(1.0, abs(fd)), (b, i, fd, grad[b, i])


@pytest.mark.parametrize('precision', ['fp32', 'split'])
def test_mft_adjoint_dot_products(precision):
    from hcipy_gb300 import _lib
    from hcipy_gb300.autograd import mft_apply
    pupil = hg.make_pupil_grid(48, 1)
    focal = hg.make_focal_grid(2.7, 6)
    ft = hg.MatrixFourierTransform(pupil, focal, precision=precision)
    rng = np.random.default_rng(3)
    tol = 1e-12 if precision == 'fp32' else 1e-8
    for direction, n_in, n_out in ((_lib.HX_FORWARD, pupil.size, focal.size),
                                   (_lib.HX_BACKWARD, focal.size, pupil.size),
                                   (_lib.HX_ADJOINT, focal.size, pupil.size)):
        x = torch.from_numpy(rng.standard_normal(n_in) + 1j * rng.standard_normal(n_in)).cuda().requires_grad_(True)
        w = torch.from_numpy(rng.standard_normal(n_out) + 1j * rng.standard_normal(n_out)).cuda()
        alpha = 0.3 - 1.7j
        y = mft_apply(ft, x, direction, alpha)
        (ahw,) = torch.autograd.grad(y, x, grad_outputs=w.to(y.dtype))
        lhs = _vdot(w, y.detach())
        rhs = _vdot(ahw, x.detach())
        scale = torch.linalg.vector_norm(w).item() * torch.linalg.vector_norm(y.detach()).item()
        assert abs(lhs - rhs) < tol * scale, (direction, lhs, rhs)


def _lyot_setup(n=64, precision='fp32'):
    from hcipy_gb300 import workloads
    pupil = hg.make_pupil_grid(n, 1)
    # q not a multiple of 1/n keeps the planner on the matrix Fourier transform (no FFT grid)
    fpm_grid = hg.make_focal_grid(3.7, 8)
    focal = hg.make_focal_grid(3.3, 10)
    fpm = 1 - workloads.circular_aperture(fpm_grid, 5.0)
    stop = workloads.circular_aperture(pupil, 0.9)
    lyot = hg.LyotCoronagraph(pupil, hg.Field(fpm, fpm_grid), hg.Field(stop, pupil), precision=precision)
    prop = hg.FraunhoferPropagator(pupil, focal, precision=precision)
    return pupil, fpm_grid, focal, fpm, stop, lyot, prop


@pytest.mark.parametrize('precision', ['fp32', 'split'])
def test_lyot_adjoint_dot_product(precision):
    pupil, _, _, _, _, lyot, _ = _lyot_setup(precision=precision)
    rng = np.random.default_rng(4)
    x = torch.from_numpy(rng.standard_normal((2, pupil.size)) + 1j * rng.standard_normal((2, pupil.size)))
    x = x.cuda().requires_grad_(True)
    w = torch.from_numpy(rng.standard_normal((2, pupil.size)) + 1j * rng.standard_normal((2, pupil.size))).cuda()
    y = lyot.forward(hg.Wavefront(hg.Field(x, pupil), 1.0)).electric_field.data
    (ahw,) = torch.autograd.grad(y, x, grad_outputs=w.to(y.dtype))
    lhs, rhs = _vdot(w, y.detach()), _vdot(ahw, x.detach())
    scale = torch.linalg.vector_norm(w).item() * torch.linalg.vector_norm(y.detach()).item()
    tol = 1e-12 if precision == 'fp32' else 1e-8
    assert abs(lhs - rhs) < tol * scale, (lhs, rhs)


def _roi(focal, r_in, r_out):
    x, y = focal.points[:, 0], focal.points[:, 1]
    r = np.hypot(x, y)
    return (r >= r_in) & (r <= r_out) & (x > 0)


@pytest.mark.parametrize('precision', ['fp32', 'split'])
def test_dm_lyot_intensity_gradient(precision):
    """Loss = sum of the image intensity over a half annulus; gradient in the actuators vs central differences
    of the float64 chain and vs the oracle loss."""
    pupil, fpm_grid, focal, fpm, stop, lyot, prop = _lyot_setup(precision=precision)
    inf = hg.make_gaussian_influence_functions(pupil, 8, 1 / 8, crosstalk=0.15)
    from hcipy_gb300 import workloads
    aperture = workloads.circular_aperture(pupil, 1.0).astype(np.complex128)
    roi = torch.from_numpy(_roi(focal, 2.0, 8.0).astype(np.float64)).cuda()
    rng = np.random.default_rng(5)
    a0 = rng.standard_normal((3, inf.num_modes)) * 2e-3
    wl = 1.0

    def loss_of(a_t, dm):
        dm.actuators = a_t
        e = dm.forward(hg.Wavefront(hg.Field(torch.from_numpy(aperture).cuda(), pupil), wl))
        img = prop.forward(lyot.forward(e)).electric_field.data
        return ((img.real**2 + img.imag**2) * roi).sum()

    dm = hg.DeformableMirror(inf, dtype=torch.float64)
    a = torch.from_numpy(a0).cuda().requires_grad_(True)
    loss = loss_of(a, dm)
    loss.backward()
    grad = a.grad.cpu().numpy()

    # oracle loss (float64 numpy chain)
    m = inf.transformation_matrix.toarray()
    chain = ooptics.LyotChain(RegularGrid(pupil.delta, pupil.dims, pupil.zero),
                              RegularGrid(fpm_grid.delta, fpm_grid.dims, fpm_grid.zero),
                              RegularGrid(focal.delta, focal.dims, focal.zero), fpm, stop)
    ref = 0.0
    for v in range(3):
        img = chain(aperture * np.exp(2j * (2 * np.pi / wl) * (m @ a0[v])))
        ref += np.sum(np.abs(img)**2 * roi.cpu().numpy())
    assert abs(loss.item() - ref) < (1e-10 if precision == 'fp32' else 1e-7) * ref

    # central differences on the float64 plain chain
    fd_prop = _lyot_setup(precision='fp32')
    h = 1e-6
    dm64 = hg.DeformableMirror(inf, dtype=torch.float64)
    for (v, i) in [(0, 5), (1, 20), (2, 40)]:
        ap = a0.copy()
        ap[v, i] += h
        am = a0.copy()
        am[v, i] -= h
        with torch.no_grad():
            lp = _loss_plain(fd_prop, dm64, ap, aperture, roi, wl)
            lm = _loss_plain(fd_prop, dm64, am, aperture, roi, wl)
        fd = (lp - lm) / (2 * h)
        tol = 1e-6 if precision == 'fp32' else 1e-5
        assert abs(fd - grad[v, i]) < tol * np.abs(grad).max(), (v, i, fd, grad[v, i])


def _loss_plain(setup, dm, a, aperture, roi, wl):
    pupil, _, _, _, _, lyot, prop = setup
    dm.actuators = torch.from_numpy(a).cuda()
    e = dm.forward(hg.Wavefront(hg.Field(torch.from_numpy(aperture).cuda(), pupil), wl))
    img = prop.forward(lyot.forward(e)).electric_field.data
    return ((img.real**2 + img.imag**2) * roi).sum().item()


@pytest.mark.parametrize('precision', ['fp32', 'split'])
def test_gradient_matches_oracle_poke_jacobian(precision):
    """The device adjoint gradient against a Jacobian built by poking actuators in the float64 oracle chain
    (central differences of the reference algorithm's loss, one actuator at a time): within 1e-6 relative."""
    pupil, fpm_grid, focal, fpm, stop, lyot, prop = _lyot_setup(n=48, precision=precision)
    inf = hg.make_gaussian_influence_functions(pupil, 6, 1 / 6, crosstalk=0.15)
    m = inf.transformation_matrix.toarray()
    from hcipy_gb300 import workloads
    aperture = workloads.circular_aperture(pupil, 1.0).astype(np.complex128)
    roi = _roi(focal, 2.0, 8.0)
    rng = np.random.default_rng(8)
    a0 = rng.standard_normal(inf.num_modes) * 2e-3
    dm = hg.DeformableMirror(inf, dtype=torch.float64)
    a = torch.from_numpy(a0).cuda().requires_grad_(True)
    dm.actuators = a
    e = dm.forward(hg.Wavefront(hg.Field(torch.from_numpy(aperture).cuda(), pupil), 1.0))
    img = prop.forward(lyot.forward(e)).electric_field.data
    loss = ((img.real**2 + img.imag**2) * torch.from_numpy(roi.astype(np.float64)).cuda()).sum()
    loss.backward()
    grad = a.grad.cpu().numpy()

    chain = ooptics.LyotChain(RegularGrid(pupil.delta, pupil.dims, pupil.zero),
                              RegularGrid(fpm_grid.delta, fpm_grid.dims, fpm_grid.zero),
                              RegularGrid(focal.delta, focal.dims, focal.zero), fpm, stop)

    def oracle_loss(act):
        img = chain(aperture * np.exp(2j * 2 * np.pi * (m @ act)))
        return np.sum(np.abs(img)**2 * roi)

    h = 1e-7
    jac = np.empty(inf.num_modes)
    for i in range(inf.num_modes):
        ap, am = a0.copy(), a0.copy()
        ap[i] += h
        am[i] -= h
        jac[i] = (oracle_loss(ap) - oracle_loss(am)) / (2 * h)
    assert np.linalg.norm(grad - jac) < 1e-6 * np.linalg.norm(jac), np.linalg.norm(grad - jac) / np.linalg.norm(jac)


def test_batch_of_one_keeps_its_dimension():
    """Commands of shape (1, nact) on an unbatched field give a (1, npix) field, as a batch of one must."""
    pupil = hg.make_pupil_grid(32, 1)
    dm = hg.DeformableMirror(hg.make_gaussian_influence_functions(pupil, 6, 1 / 6))
    e = torch.ones(pupil.size, dtype=torch.complex64, device='cuda')
    cmd = torch.full((1, dm.num_actuators), 1e-3, device='cuda')
    dm.actuators = cmd
    out = dm.forward(hg.Wavefront(hg.Field(e, pupil), 1.0)).electric_field.data
    assert out.shape == (1, pupil.size)
    dm.actuators = cmd[0]
    single = dm.forward(hg.Wavefront(hg.Field(e, pupil), 1.0)).electric_field.data
    assert single.shape == (pupil.size,) and torch.equal(single, out[0])


@pytest.mark.parametrize('dtype,tol', [(torch.float64, 1e-12), (torch.float32, 2e-6)])
def test_sparse_basis_staged_and_blocked_paths(dtype, tol):
    """The surface kernel stages each CTA's actuator range of the commands in shared memory and the transpose
    walks blocks of 4 actuators: against float64 dense products for 37 vectors (ragged against the 16 / 8
    vectors a CTA takes), 1001 actuators (a ragged last block), a banded basis (staged) and one whose rows
    reach across all actuators (too wide to stage: the global path).  The CSC transpose gives the same result,
    and the surface is right for unsorted CSR columns at the C ABI."""
    import scipy.sparse as sp
    from hcipy_gb300 import _lib
    from hcipy_gb300.kernels import SparseBasis
    rng = np.random.default_rng(4)
    npix, nact, nvec = 3000, 1001, 37
    rows, cols = [], []
    for p in range(npix):  # banded: pixel p touches actuators near p / 3
        c = np.unique(np.clip(p // 3 + rng.integers(-20, 21, 12), 0, nact - 1))
        rows += [p] * c.size
        cols += list(c)
    banded = sp.csr_matrix((rng.standard_normal(len(rows)), (rows, cols)), shape=(npix, nact))
    wide = sp.random(npix, nact, density=0.02, random_state=5, format='csr')
    for m in (banded, wide):
        basis = SparseBasis(m, torch.device('cuda'), dtype)
        a = rng.standard_normal((nvec, nact))
        s = basis.apply(torch.from_numpy(a)).double().cpu().numpy()
        ref = a @ m.T.toarray()
        assert rel_err(s, ref) < tol
        w = rng.standard_normal((nvec, npix))
        gt = basis.apply_transpose(torch.from_numpy(w)).double().cpu().numpy()
        assert rel_err(gt, w @ m.toarray()) < tol
        g2 = torch.from_numpy(w).to('cuda', dtype)
        out = torch.empty((nvec, nact), dtype=dtype, device='cuda')
        rc = _lib.lib().hx_influence_apply_transpose(npix, nact, _lib.dptr(basis.col_ptr), _lib.dptr(basis.row_idx),
                                                     _lib.dptr(basis.vals_csc), _lib.dtype_code(dtype), nvec,
                                                     _lib.dptr(g2), _lib.dptr(out), _lib.stream_handle())
        _lib.check(rc)
        assert rel_err(out.double().cpu().numpy(), gt) < tol
    # unsorted columns within each CSR row
    m = banded.copy()
    perm = np.concatenate([rng.permutation(np.arange(m.indptr[p], m.indptr[p + 1])) for p in range(npix)])
    idx = torch.from_numpy(m.indices[perm].astype(np.int32)).cuda()
    val = torch.from_numpy(m.data[perm]).to('cuda', dtype)
    ptr = torch.from_numpy(m.indptr.astype(np.int32)).cuda()
    a = rng.standard_normal((nvec, nact))
    a_dev = torch.from_numpy(a).to('cuda', dtype)
    out = torch.empty((nvec, npix), dtype=dtype, device='cuda')
    _lib.check(_lib.lib().hx_influence_apply(npix, nact, _lib.dptr(ptr), _lib.dptr(idx), _lib.dptr(val),
                                             _lib.dtype_code(dtype), nvec, _lib.dptr(a_dev), _lib.dptr(out),
                                             _lib.stream_handle()))
    assert rel_err(out.double().cpu().numpy(), a @ m.T.toarray()) < tol
