"""Multi-scale vortex coronagraph against the reference's own propagation (golden vectors from
hcipy/coronagraphy/vortex.py and multi_scale.py): the level masks built on the device, the Lyot-plane field of an
aberrated pupil and the backward propagation of a random field.
Tolerances: complex128 1e-10 relative (float64 FFTs and GEMMs in another order); complex64 fields 2e-5 (a few
float32 transforms summed over the levels).
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


@pytest.mark.parametrize('case', ['vortex_0', 'vortex_1'])
def test_vortex_matches_reference(case):
    g = load_golden(case)
    pupil = hg.make_pupil_grid(int(g['n']), 1.0)
    vc = hg.VortexCoronagraph(pupil, int(g['charge']), q=int(g['q']), scaling_factor=int(g['scaling_factor']),
                              window_size=int(g['window_size']))
    assert len(vc.focal_masks) == int(g['levels'])
    for k, m in enumerate(vc.focal_masks):
        assert rel_err(m.numpy(), g['mask_%d' % k]) < 1e-10, k
    lyot = vc.forward(hg.Wavefront(hg.Field(g['E'], pupil), 1.0)).electric_field.numpy()
    assert rel_err(lyot, g['lyot_c128']) < 1e-10
    back = vc.backward(hg.Wavefront(hg.Field(g['G'], pupil), 1.0)).electric_field.numpy()
    assert rel_err(back, g['back_c128']) < 1e-10
    lyot32 = vc.forward(hg.Wavefront(hg.Field(g['E'].astype(np.complex64), pupil), 1.0)).electric_field.numpy()
    assert lyot32.dtype == np.complex64 and rel_err(lyot32, g['lyot_c128']) < 2e-5


def test_vortex_batch_and_lyot_stop():
    """A batch of fields is one set of launches per level; a Lyot stop multiplies the result."""
    g = load_golden('vortex_1')
    pupil = hg.make_pupil_grid(int(g['n']), 1.0)
    stop = hg.Field((np.hypot(*pupil.points_list()) <= 0.45).astype(np.float64), pupil)
    vc = hg.VortexCoronagraph(pupil, int(g['charge']), lyot_stop=stop, q=int(g['q']),
                              scaling_factor=int(g['scaling_factor']), window_size=int(g['window_size']))
    e = torch.from_numpy(np.stack([g['E'], g['G']])).cuda()
    out = vc.forward(hg.Wavefront(hg.Field(e, pupil), 1.0)).electric_field.numpy()
    assert rel_err(out[0], g['lyot_c128'] * stop.numpy()) < 1e-10
    single = vc.forward(hg.Wavefront(hg.Field(g['G'], pupil), 1.0)).electric_field.numpy()
    assert rel_err(out[1], single) < 1e-12


def test_lazy_conjugate_views_are_materialised():
    """torch's conj() only flags a view; a field or mask passed that way reaches the kernels conjugated."""
    pupil = hg.make_pupil_grid(32, 1.0)
    focal = hg.make_focal_grid(3.3, 5)
    mft = hg.MatrixFourierTransform(pupil, focal)
    rng = np.random.default_rng(2)
    e = torch.from_numpy(rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)).cuda()
    ref = mft.forward(e.conj().resolve_conj()).numpy()
    assert rel_err(mft.forward(e.conj()).numpy(), ref) < 1e-14
    m = torch.from_numpy(np.exp(1j * rng.standard_normal(focal.size))).cuda()
    from hcipy_gb300 import _lib
    out = mft._run(e, mft.input_grid, mft.output_grid, _lib.HX_FORWARD, complex(mft._w_in_scalar),
                   epilogue=_lib.HX_EPI_MUL, mask=m.conj()).numpy()
    assert rel_err(out, mft.forward(e).numpy() * np.conj(m.cpu().numpy())) < 1e-12


def _vector_vortex(g, stop=True):
    pupil = hg.make_pupil_grid(48, 1.0)
    return pupil, hg.VectorVortexCoronagraph(2, lyot_stop=hg.Field(g['stop'], pupil) if stop else None,
                                             phase_retardation=lambda wl: np.pi * (1 + 0.05 * (wl - 1)), q=32,
                                             scaling_factor=2, window_size=16)


def test_vector_vortex_matches_reference():
    """VectorVortexCoronagraph (hcipy/coronagraphy/vortex.py:17-246) against the reference: the Lyot-plane Jones
    matrix of an unpolarised pupil at two wavelengths (a chromatic retardance) and the Stokes parameters of its image
    through a lens (the polarised wavefront's I/Q/U/V, wavefront.py:103-255); a partially polarised input; backward
    of a Jones-matrix field and of a scalar field; complex64.  Tolerances: fields 1e-10, Stokes parameters 1e-9
    (complex128); complex64 2e-5."""
    g = load_golden('vector_vortex')
    pupil, vvc = _vector_vortex(g)
    prop = hg.FraunhoferPropagator(pupil, hg.make_focal_grid(4, 8))
    for k in range(2):
        wl = float(g['wavelength_%d' % k])
        lyot = vvc.forward(hg.Wavefront(hg.Field(g['E'], pupil), wl))
        assert lyot.is_polarized and lyot.wavelength == wl
        assert np.array_equal(lyot.input_stokes_vector, g['lyot_stokes_%d' % k])
        assert rel_err(lyot.electric_field.numpy(), g['lyot_%d' % k]) < 1e-10, k
        img = prop(lyot)
        assert img.is_polarized
        iquv = np.stack([img.I.numpy(), img.Q.numpy(), img.U.numpy(), img.V.numpy()])
        assert rel_err(iquv, g['image_%d' % k]) < 1e-9, k
        assert rel_err(img.stokes_vector.numpy(), g['image_%d' % k]) < 1e-9
    assert len(vvc._entries) == 2  # one set of three scalar coronagraphs per retardance
    pol = vvc.forward(hg.Wavefront(hg.Field(g['EJ'], pupil), 1.0, g['stokes']))
    assert np.array_equal(pol.input_stokes_vector, g['stokes'])
    assert rel_err(pol.electric_field.numpy(), g['lyot_pol']) < 1e-10
    assert rel_err(pol.stokes_vector.numpy(), g['lyot_pol_stokes']) < 1e-9
    back = vvc.backward(hg.Wavefront(hg.Field(g['G'], pupil), 1.0, g['stokes']))
    assert rel_err(back.electric_field.numpy(), g['back']) < 1e-10
    back = vvc.backward(hg.Wavefront(hg.Field(g['G'][0, 0], pupil), 1.0))
    assert rel_err(back.electric_field.numpy(), g['back_scalar']) < 1e-10
    _, bare = _vector_vortex(g, stop=False)
    lyot32 = bare.forward(hg.Wavefront(hg.Field(g['E'].astype(np.complex64), pupil), 1.0)).electric_field.numpy()
    assert lyot32.dtype == np.complex64 and rel_err(lyot32 * g['stop'], g['lyot_0']) < 2e-5
    with pytest.raises(ValueError):
        vvc.forward(hg.Wavefront(hg.Field(np.stack([g['E'], g['E']]), pupil), 1.0))


def test_polarised_wavefront_stokes_parameters():
    """A scalar field with a Stokes vector becomes E times the identity, whose Stokes parameters are |E|^2 times the
    input vector; a scalar wavefront is unpolarised (Q = U = V = 0); elements keep the input Stokes vector."""
    pupil = hg.make_pupil_grid(16, 1.0)
    rng = np.random.default_rng(3)
    e = rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)
    s = np.array([1.0, 0.4, -0.3, 0.2])
    wf = hg.Wavefront(hg.Field(e, pupil), 1.0, s)
    j = wf.electric_field.numpy()
    assert j.shape == (2, 2, pupil.size)
    assert np.array_equal(j[0, 0], e) and np.array_equal(j[1, 1], e) and not j[0, 1].any() and not j[1, 0].any()
    ref = np.abs(e)**2 * s[:, np.newaxis]
    assert rel_err(wf.stokes_vector.numpy(), ref) < 1e-15
    assert rel_err(wf.power.numpy(), ref[0] * pupil.weights) < 1e-15
    dop = wf.degree_of_polarization.numpy()
    assert np.allclose(dop, np.sqrt(0.4**2 + 0.3**2 + 0.2**2), rtol=1e-14)
    out = hg.Apodizer(hg.Field(np.ones(pupil.size) * 0.5, pupil)).forward(wf)
    assert np.array_equal(out.input_stokes_vector, s) and rel_err(out.I.numpy(), 0.25 * ref[0]) < 1e-15
    scalar = hg.Wavefront(hg.Field(e, pupil), 1.0)
    assert scalar.is_scalar and not scalar.Q.numpy().any()
    assert rel_err(scalar.stokes_vector.numpy()[0], np.abs(e)**2) < 1e-15
    with pytest.raises(ValueError):
        hg.Wavefront(hg.Field(np.stack([e, e, e]), pupil), 1.0, s)
