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
