"""Empty batches: a tensor field with a leading dimension of 0 passes through every operator and comes back
empty with the right shape (the reference loops over the batch and does nothing); the transforms launch nothing."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


@pytest.mark.parametrize('precision', ['fp32', 'split'])
def test_empty_batches_through_the_operators(precision):
    pupil = hg.make_pupil_grid(64, 1)
    focal = hg.make_focal_grid(4, 8)
    e0 = torch.empty((0, pupil.size), dtype=torch.complex64, device='cuda')
    before = hg.launch_count()
    mft = hg.MatrixFourierTransform(pupil, focal.scaled(2 * np.pi), precision=precision)
    assert tuple(mft.forward(hg.Field(e0, pupil)).data.shape) == (0, focal.size)
    assert tuple(mft.backward(hg.Field(torch.empty((0, focal.size), dtype=torch.complex64, device='cuda'),
                                       focal)).data.shape) == (0, pupil.size)
    prop = hg.FraunhoferPropagator(pupil, focal, precision=precision)
    assert tuple(prop.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0)).electric_field.data.shape) == (0, focal.size)
    assert hg.launch_count() == before  # no plan was built and nothing ran on the device
    fpm_grid = hg.make_focal_grid(8, 4)
    fpm = 1 - np.hypot(*fpm_grid.points_list()).__le__(2).astype(float)
    lyot = hg.LyotCoronagraph(pupil, hg.Field(fpm, fpm_grid), precision=precision)
    assert tuple(lyot.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0)).electric_field.data.shape) == (0, pupil.size)
    fft = hg.FastFourierTransform(pupil, q=2)
    assert tuple(fft.forward(hg.Field(e0, pupil)).data.shape) == (0, fft.output_grid.size)
    asp = hg.AngularSpectrumPropagator(pupil, 0.1)
    assert tuple(asp.forward(hg.Wavefront(hg.Field(e0, pupil), 1e-6)).electric_field.data.shape) == (0, pupil.size)
    czt = hg.ChirpZTransform(64, 32, np.exp(-2j * np.pi / 64), 1.0)
    assert tuple(czt(torch.empty((0, 64), dtype=torch.complex64, device='cuda')).shape) == (0, 32)
    dm = hg.DeformableMirror(hg.make_gaussian_influence_functions(pupil, 6, 1 / 6))
    dm.actuators = torch.empty((0, dm.num_actuators), device='cuda')
    assert tuple(dm.surface.data.shape) == (0, pupil.size)
    one = torch.ones(pupil.size, dtype=torch.complex64, device='cuda')
    assert tuple(dm.forward(hg.Wavefront(hg.Field(one, pupil), 1.0)).electric_field.data.shape) == (0, pupil.size)
