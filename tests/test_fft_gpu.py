"""Parity of the device FFT family with the reference's golden vectors and the float64 oracle.

Tolerances (relative L2 error of the whole field unless stated):
  complex128 (float64 FFT on the device)   : 1e-11
  complex64  (float32 FFT)                  : 2e-6
  chirp-Z, as the reference's own test      : rtol 1e-10 (complex128, our chirp is computed
                                              independently of numpy's power), 1e-4 (complex64)
"""
import numpy as np
import pytest
import torch

from conftest import load_golden, grid_from, rel_err
from oracle import fourier as ofourier, grids as ogrids

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')


def regular(g, prefix):
    return hg.CartesianGrid(hg.RegularCoords(g[prefix + '_delta'], g[prefix + '_dims'], g[prefix + '_zero']))


@pytest.mark.parametrize('case', ['fft_0', 'fft_1', 'fft_2', 'fft_3'])
@pytest.mark.parametrize('dtype', ['complex128', 'complex64'])
def test_fft_matches_reference(case, dtype):
    g = load_golden(case)
    pupil = regular(g, 'ingrid')
    fft = hg.FastFourierTransform(pupil, q=float(g['q']), fov=float(g['fov']), shift=tuple(g['shift']))
    np.testing.assert_array_equal(fft.output_grid.dims, g['outgrid_dims'])
    fwd = fft.forward(g['E'].astype(dtype)).numpy()
    bwd = fft.backward(g['F'].astype(dtype)).numpy()
    tol = 1e-11 if dtype == 'complex128' else 2e-6
    assert rel_err(fwd, g['fwd_exact_c128']) < tol
    assert rel_err(bwd, g['bwd_c128']) < tol


@pytest.mark.parametrize('dims,q,fov', [((30, 42), 1.5, 1), ((17, 13), 1, 1), ((21, 10), 2, 0.7), ((64, 1), 2, 1)])
def test_fft_mixed_radix_and_bluestein(dims, q, fov):
    """Padded lengths with factors 3, 5, 7 (mixed radix) and 17, 13 (Bluestein)."""
    rng = np.random.default_rng(7)
    pupil = hg.make_pupil_grid(dims, 1.3)
    fft = hg.FastFourierTransform(pupil, q=q, fov=fov, shift=(0.2, -0.1))
    ogrid = ogrids.RegularGrid(pupil.delta, pupil.dims, pupil.zero)
    plan = ofourier.FFTPlan(ogrid, q, fov, (0.2, -0.1))
    e = rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)
    f = rng.standard_normal(fft.output_grid.size) + 1j * rng.standard_normal(fft.output_grid.size)
    assert rel_err(fft.forward(e).numpy(), plan.forward(e)) < 1e-11
    assert rel_err(fft.backward(f).numpy(), plan.backward(f)) < 1e-11
    assert rel_err(fft.forward(e.astype(np.complex64)).numpy(), plan.forward(e)) < 2e-6


def test_fft_cfg2_size_and_round_trip():
    """1024^2 pupil zero-padded to 4096^2 (q=4), complex64, against the float64 oracle; energy and round trip."""
    rng = np.random.default_rng(8)
    pupil = hg.make_pupil_grid(1024, 8.0)
    fft = hg.FastFourierTransform(pupil, q=4)
    e = (rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)).astype(np.complex64)
    out = fft.forward(e)
    assert out.shape == (4096 * 4096,)
    ref = ofourier.FFTPlan(ogrids.RegularGrid(pupil.delta, pupil.dims, pupil.zero), 4).forward(e.astype(complex))
    assert rel_err(out.numpy(), ref) < 2e-6
    back = fft.backward(out).numpy()
    assert rel_err(back, e) < 2e-6
    # Parseval with the grid weights.
    e_in = np.sum(np.abs(e.astype(complex))**2) * pupil.weights
    e_out = np.sum(np.abs(out.numpy().astype(complex))**2) * fft.output_grid.weights / (2 * np.pi)**2
    assert abs(e_out / e_in - 1) < 1e-5


@pytest.mark.parametrize('dims,q,shift', [((40, 256), 2, (0.0, 0.0)), ((8, 256), 4, (0.3, -0.2)),
                                           ((16, 128), 8, (0.0, 0.25)), ((16, 256), 16, (0.0, 0.0)),
                                           ((12, 1024), 4, (-0.2, 0.1)), ((8, 512), 4, (0.0, 0.0)),
                                           ((8, 1536), 8 / 3, (0.0, 0.1)), ((8, 384), 8 / 3, (0.0, 0.0)),
                                           ((8, 768), 8 / 3, (0.2, 0.0)), ((8, 200), 10.24, (0.0, -0.3)),
                                           ((8, 500), 8.192, (0.0, 0.0))])
def test_fft_zero_padded_power_of_two_columns(dims, q, shift):
    """complex64 transforms zero-padded along y to a power of two of 512-4096 points (the register-resident line
    kernel on strided columns) with 1/2 to 1/16 of each column valid, shifted grids, forward and backward, against
    the float64 oracle."""
    rng = np.random.default_rng(dims[1] + int(10 * q))
    pupil = hg.make_pupil_grid(dims, (1.0, 2.0))
    fft = hg.FastFourierTransform(pupil, q=q, shift=shift)
    plan = ofourier.FFTPlan(ogrids.RegularGrid(pupil.delta, pupil.dims, pupil.zero), q, 1, shift)
    e = (rng.standard_normal(pupil.size) + 1j * rng.standard_normal(pupil.size)).astype(np.complex64)
    f = (rng.standard_normal(fft.output_grid.size) + 1j * rng.standard_normal(fft.output_grid.size)).astype(np.complex64)
    assert rel_err(fft.forward(e).numpy(), plan.forward(e.astype(complex))) < 2e-6
    assert rel_err(fft.backward(f).numpy(), plan.backward(f.astype(complex))) < 2e-6


def test_fft_tensor_field_batches():
    rng = np.random.default_rng(9)
    pupil = hg.make_pupil_grid(24, 1)
    fft = hg.FastFourierTransform(pupil, q=2, fov=0.5)
    e = rng.standard_normal((2, 3, pupil.size)) + 1j * rng.standard_normal((2, 3, pupil.size))
    res = fft.forward(e).numpy()
    for i in range(2):
        for j in range(3):
            assert rel_err(res[i, j], fft.forward(e[i, j]).numpy()) < 1e-13


def test_czt_matches_reference():
    g = load_golden('czt')
    for i in range(4):
        x, w, a, m = g['x_%d' % i], complex(g['w_%d' % i]), complex(g['a_%d' % i]), int(g['m_%d' % i])
        czt = hg.ChirpZTransform(len(x), m, w, a)
        y = czt(x).cpu().numpy()
        np.testing.assert_allclose(y, g['y_%d' % i], rtol=1e-10, atol=1e-10 * np.abs(g['y_%d' % i]).max())
        y64 = czt(x.astype(np.complex64)).cpu().numpy()
        assert y64.dtype == np.complex64
        assert rel_err(y64, g['y_%d' % i]) < 1e-4
    czt = hg.ChirpZTransform(19, 31, np.exp(-0.2j), np.exp(0.7j))
    assert rel_err(czt(g['xb']).cpu().numpy(), g['yb']) < 1e-12


def test_zoomfft_matches_reference():
    g = load_golden('zoomfft')
    gi, go = regular(g, 'ingrid'), regular(g, 'outgrid')
    zfft = hg.ZoomFastFourierTransform(gi, go)
    assert rel_err(zfft.forward(g['E']).numpy(), g['fwd_c128']) < 1e-11
    assert rel_err(zfft.backward(g['F']).numpy(), g['bwd_c128']) < 1e-11
    assert rel_err(zfft.forward(g['E'].astype(np.complex64)).numpy(), g['fwd_c128']) < 1e-5
    # ZoomFFT, MFT and the reference agree.
    mft = hg.MatrixFourierTransform(gi, go)
    assert rel_err(mft.forward(g['E']).numpy(), zfft.forward(g['E']).numpy()) < 1e-11


def test_fourier_filter_matches_reference():
    g = load_golden('fourier_filter')
    gi = regular(g, 'ingrid')
    ff = hg.FourierFilter(gi, g['tf'], q=2)
    assert rel_err(ff.forward(g['E']).numpy(), g['fwd_c128']) < 1e-12
    assert rel_err(ff.backward(g['E']).numpy(), g['bwd_c128']) < 1e-12
    assert rel_err(ff.forward(g['E'].astype(np.complex64)).numpy(), g['fwd_c128']) < 2e-6


@pytest.mark.parametrize('case', ['asp_0', 'asp_1', 'asp_2', 'asp_3'])
def test_angular_spectrum_matches_reference(case):
    g = load_golden(case)
    pupil = hg.make_pupil_grid(int(g['n']), float(g['diam']))
    asp = hg.AngularSpectrumPropagator(pupil, float(g['distance']))
    wl = float(g['wavelength'])
    out = asp.forward(hg.Wavefront(hg.Field(g['E'], pupil), wl)).electric_field.numpy()
    # The transfer-function phase k_z d reaches ~1e7 rad; float64 rounding of that product differs by ~1e-9 rad.
    assert rel_err(out, g['fwd_c128']) < 1e-8
    back = asp.backward(hg.Wavefront(hg.Field(g['fwd_c128'], pupil), wl)).electric_field.numpy()
    assert rel_err(back, g['bwd_c128']) < 1e-8
    out64 = asp.forward(hg.Wavefront(hg.Field(g['E'].astype(np.complex64), pupil), wl)).electric_field.numpy()
    assert rel_err(out64, g['fwd_c128']) < 5e-6


@pytest.mark.parametrize('case', ['fresnel_0', 'fresnel_1', 'fresnel_2', 'fresnel_3', 'fresnel_4'])
def test_fresnel_matches_reference(case):
    """FresnelPropagator against the reference's propagation: both transfer-function branches, zero padding 2
    and 3, refractive index 1 and 1.5; forward, backward and complex64 fields."""
    g = load_golden(case)
    pupil = hg.make_pupil_grid(int(g['n']), float(g['diam']))
    prop = hg.FresnelPropagator(pupil, float(g['distance']), zero_padding=int(g['zero_padding']),
                                refractive_index=float(g['refractive_index']))
    wl = float(g['wavelength'])
    out = prop.forward(hg.Wavefront(hg.Field(g['E'], pupil), wl)).electric_field.numpy()
    # The phase k d reaches ~2e10 rad at 5 km; its float64 rounding differs from the reference's by ~1e-9 rad.
    assert rel_err(out, g['fwd_c128']) < 1e-8
    back = prop.backward(hg.Wavefront(hg.Field(g['fwd_c128'], pupil), wl)).electric_field.numpy()
    assert rel_err(back, g['bwd_c128']) < 1e-8
    out64 = prop.forward(hg.Wavefront(hg.Field(g['E'].astype(np.complex64), pupil), wl)).electric_field.numpy()
    assert out64.dtype == np.complex64 and rel_err(out64, g['fwd_c128']) < 5e-6


def test_planner_choices():
    """The default planner makes the reference's choices (hcipy tests/test_fourier.py planner cases, with the
    reference's own cost model): an FFT for a 128^2 pupil at q=1, an MFT at q=8 fov=0.3, a zoom FFT for 1024^2 at
    q=8 fov=0.1.  The GB300 cost model and the measuring planner return valid operators."""
    pupil = hg.make_pupil_grid(128)
    assert isinstance(hg.make_fourier_transform(pupil, q=1, fov=1), hg.FastFourierTransform)
    assert isinstance(hg.make_fourier_transform(pupil, q=8, fov=0.3), hg.MatrixFourierTransform)
    assert isinstance(hg.make_fourier_transform(hg.make_pupil_grid(1024), q=8, fov=0.1), hg.ZoomFastFourierTransform)
    assert isinstance(hg.make_fourier_transform(pupil, q=2, fov=1, planner='gpu'), hg.FourierTransform)
    assert isinstance(hg.make_fourier_transform(pupil, q=2, fov=1, planner='measure'), hg.FourierTransform)
    with pytest.raises(ValueError):
        hg.make_fourier_transform(pupil, q=2, planner='guess')
