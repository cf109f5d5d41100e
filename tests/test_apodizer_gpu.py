"""Thin apodizers on the device against the float64 oracle (hcipy/optics/apodization.py:6-62).

Tolerances: complex128 fields 1e-13 relative (one complex product, exp in float64 on both sides); complex64
fields 1e-6 (the phase factor in float32).
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import optics as ooptics

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


@pytest.mark.parametrize('dtype,tol', [(np.complex128, 1e-13), (np.complex64, 1e-6)])
def test_phase_apodizer_forward_backward(dtype, tol):
    grid = hg.make_pupil_grid(37, 1.0)
    rng = np.random.default_rng(31)
    phase = rng.uniform(-np.pi, np.pi, grid.size)
    e = (rng.standard_normal((3, grid.size)) + 1j * rng.standard_normal((3, grid.size))).astype(dtype)
    apod = hg.PhaseApodizer(hg.Field(phase, grid))
    wf = hg.Wavefront(hg.Field(e, grid), 0.8)
    out = apod.forward(wf).electric_field.numpy()
    assert out.dtype == dtype and out.shape == e.shape
    ref = ooptics.apodize(e.astype(complex), np.exp(1j * phase))
    assert rel_err(out, ref) < tol
    back = apod.backward(wf).electric_field.numpy()
    assert rel_err(back, ooptics.apodize(e.astype(complex), np.exp(1j * phase), adjoint=True)) < tol
    round_trip = apod.backward(apod.forward(wf)).electric_field.numpy()
    assert rel_err(round_trip, e.astype(complex)) < tol
    assert np.array_equal(apod.phase.numpy(), phase)


def test_phase_apodizer_scalar_phase():
    grid = hg.make_pupil_grid(16, 1.0)
    rng = np.random.default_rng(4)
    e = rng.standard_normal(grid.size) + 1j * rng.standard_normal(grid.size)
    wf = hg.Wavefront(hg.Field(e, grid), 1.0)
    out = hg.PhaseApodizer(0.3).forward(wf).electric_field.numpy()
    assert rel_err(out, e * np.exp(0.3j)) < 1e-13
    out = hg.PhaseApodizer(0.3).backward(wf).electric_field.numpy()
    assert rel_err(out, e * np.exp(-0.3j)) < 1e-13


def test_apodizer_complex_and_batched():
    grid = hg.make_pupil_grid(29, 1.0)
    rng = np.random.default_rng(6)
    a = rng.standard_normal(grid.size) + 1j * rng.standard_normal(grid.size)
    e = rng.standard_normal((2, grid.size)) + 1j * rng.standard_normal((2, grid.size))
    apod = hg.Apodizer(hg.Field(a, grid))
    wf = hg.Wavefront(hg.Field(e, grid), 1.0)
    assert rel_err(apod.forward(wf).electric_field.numpy(), ooptics.apodize(e, a)) < 1e-14
    assert rel_err(apod.backward(wf).electric_field.numpy(), ooptics.apodize(e, a, adjoint=True)) < 1e-14
