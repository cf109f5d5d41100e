"""Seeded synthetic inputs of the benchmark configurations (host-side, float64 numpy).

Stand-ins for the reference's input generators, with the same shapes and value
distributions: a circular aperture (hcipy/aperture/generic.py:11-46), Noll-indexed
Zernike modes on the unit disk (hcipy/mode_basis/zernike.py:455-506) and
random coefficients scaled to a stated RMS inside the aperture.  These run once
per workload on the host; the propagation itself runs on the device.
"""
import math

import numpy as np

from .field import make_pupil_grid, make_focal_grid


def mft_complex_macs(nx, ny, nu, nv):
    """Complex multiply-accumulates of one matrix Fourier transform (ny x nx) -> (nv x nu) as two GEMMs,
    E . M2 then M1 . (E M2) (the order of hcipy/fourier/matrix_fourier_transform.py:282-292)."""
    return ny * nx * nu + nv * ny * nu


def broadband_turbulence_workload(pupil_n=1024, diameter=8.0, num_wavelengths=21, bandwidth=0.2, q=4,
                                  num_airy=32, reference_wavelength=500e-9,
                                  layers=((0.1, 10.0, 0.0, 5), (0.2, 15.0, 0.0, 6), (0.3, 25.0, 0.0, 7)), L0=25.0,
                                  frame_time=1e-3):  # noqa: N803
    """Broadband imaging through a three-layer frozen-flow atmosphere.

    A ``pupil_n``^2 pupil of ``diameter`` meters; ``num_wavelengths`` wavelengths spanning ``bandwidth`` around
    ``reference_wavelength``, each imaged on its own diffraction-scaled focal grid (q samples per
    lambda0/D, num_airy lambda0/lambda radius, in lambda0/D units, so the focal length is D / lambda0); layers
    given as (r0 in m at 500 nm, wind speed m/s, wind direction deg, seed), outer scale ``L0`` m, frames
    ``frame_time`` s apart.  Returns the grids and parameters; the layers themselves are built by the caller
    (they need the GPU)."""
    from .broadband import diffraction_scaled_focal_grids
    pupil = make_pupil_grid(pupil_n, diameter)
    rel = np.linspace(1 - bandwidth / 2, 1 + bandwidth / 2, num_wavelengths)
    return {
        'pupil': pupil,
        'aperture': circular_aperture(pupil, diameter),
        'wavelengths': rel * reference_wavelength,
        'focal_grids': diffraction_scaled_focal_grids(q, num_airy, rel, 1.0),
        'focal_length': diameter / reference_wavelength,
        'layers': [{'r0': r0, 'velocity': (v * math.cos(math.radians(a)), v * math.sin(math.radians(a))),
                    'seed': seed} for r0, v, a, seed in layers],
        'L0': L0,
        'frame_time': frame_time,
    }


def circular_aperture(grid, diameter, center=(0.0, 0.0)):
    """1 inside the circle of ``diameter`` (boundary inclusive), else 0, as in generic.py:31-44."""
    x, y = grid.points_list()
    return ((x - center[0])**2 + (y - center[1])**2 <= (diameter / 2)**2).astype(np.float64)


def noll_to_zernike(j):
    """Noll index (1-based) -> (n, m)."""
    n = 0
    j1 = j - 1
    while j1 > n:
        n += 1
        j1 -= n
    m = (-1)**j * ((n % 2) + 2 * int((j1 + ((n + 1) % 2)) / 2))
    return n, m


def zernike(n, m, r, theta):
    """Orthonormal (unit RMS over the unit disk) Zernike polynomial."""
    mm = abs(m)
    rad = np.zeros_like(r)
    for k in range((n - mm) // 2 + 1):
        c = (-1)**k * math.factorial(n - k) / (math.factorial(k) * math.factorial((n + mm) // 2 - k)
                                                * math.factorial((n - mm) // 2 - k))
        rad += c * r**(n - 2 * k)
    if m == 0:
        return math.sqrt(n + 1) * rad
    if m > 0:
        return math.sqrt(2 * (n + 1)) * rad * np.cos(mm * theta)
    return math.sqrt(2 * (n + 1)) * rad * np.sin(mm * theta)


def zernike_phase(grid, diameter, first, last, rms, seed):
    """sum_{j=first..last} c_j Z_j with c ~ N(0,1), scaled to ``rms`` inside the aperture."""
    x, y = grid.points_list()
    r = np.hypot(x, y) / (diameter / 2)
    theta = np.arctan2(y, x)
    rng = np.random.default_rng(seed)
    coeffs = rng.standard_normal(last - first + 1)
    phase = np.zeros_like(r)
    for c, j in zip(coeffs, range(first, last + 1)):
        n, m = noll_to_zernike(j)
        phase += c * zernike(n, m, r, theta)
    inside = r <= 1
    phase -= phase[inside].mean()
    phase *= rms / np.std(phase[inside])
    return phase


def lyot_workload(pupil_n=2048, fpm_q=8, fpm_num_airy=32, occulter_radius=4.0, stop_diameter=0.9,
                  final_q=8, final_num_airy=32, rms_rad=2 * np.pi * 1e-3, seed=3, nmodes=(2, 100)):
    """The precision-form coronagraph workload: aberrated circular pupil, occulting FPM, Lyot stop.

    Defaults: 2048^2 pupil, FPM radius 4 lambda/D on a q=8, num_airy=32 grid
    (512^2), Lyot stop 0.9 D, final focal grid q=8, num_airy=32 (512^2),
    Zernike 2-100 at 1 nm RMS (2 pi 1e-3 rad at lambda0 = 1 um).
    """
    pupil = make_pupil_grid(pupil_n, 1)
    aperture = circular_aperture(pupil, 1.0)
    phase = zernike_phase(pupil, 1.0, nmodes[0], nmodes[1], rms_rad, seed)
    e = aperture * np.exp(1j * phase)
    fpm_grid = make_focal_grid(fpm_q, fpm_num_airy)
    fpm = 1 - circular_aperture(fpm_grid, 2 * occulter_radius)
    stop = circular_aperture(pupil, stop_diameter)
    focal = make_focal_grid(final_q, final_num_airy)
    return dict(pupil=pupil, aperture=aperture, E=e, fpm_grid=fpm_grid, fpm=fpm, stop=stop, focal=focal)


def fraunhofer_workload(pupil_n=256, q=4, num_airy=16, rms_rad=0.1, seed=0):
    """Small Fraunhofer propagation: a ``pupil_n``^2 circular pupil with Zernike 2-21 aberrations at ``rms_rad`` RMS
    (seed 0) onto a q=4, num_airy=16 focal grid (128^2)."""
    pupil = make_pupil_grid(pupil_n, 1)
    aperture = circular_aperture(pupil, 1.0)
    e = aperture * np.exp(1j * zernike_phase(pupil, 1.0, 2, 21, rms_rad, seed))
    return dict(pupil=pupil, aperture=aperture, E=e, focal=make_focal_grid(q, num_airy))


def turbulent_pupil_workload(pupil_n=1024, diameter=8.0, r0=0.15, L0=20.0, wavelength=1.6e-6, seed=1):  # noqa: N803
    """A ``pupil_n``^2 circular pupil of ``diameter`` m behind a von Karman phase screen (r0 at 500 nm, outer
    scale L0) seen at ``wavelength``: the input of the padded-FFT and angular-spectrum workloads."""
    from .atmosphere import Cn_squared_from_fried_parameter, von_karman_screen
    pupil = make_pupil_grid(pupil_n, diameter)
    aperture = circular_aperture(pupil, diameter)
    rng = np.random.default_rng(seed)
    screen = von_karman_screen(pupil_n, pupil_n, np.asarray(pupil.delta, np.float64),
                               Cn_squared_from_fried_parameter(r0, 500e-9), L0, rng)
    e = aperture * np.exp(1j * np.asarray(screen).ravel() / wavelength)
    return dict(pupil=pupil, aperture=aperture, E=e, wavelength=wavelength)


def dark_hole_mask(focal, r_in=3.0, r_out=15.0):
    x, y = focal.points_list()
    r = np.hypot(x, y)
    return (r >= r_in) & (r <= r_out)


def dm_gradient_workload(pupil_n=512, n_act=34, crosstalk=0.15, nvec=64, act_rms=1e-3, seed=4, fpm_q=8,
                         fpm_num_airy=32, occulter_radius=4.0, stop_diameter=0.9, final_q=4, final_num_airy=32,
                         roi=(3.0, 12.0)):
    """The adjoint-gradient workload: a Gaussian-influence DM ahead of the Lyot coronagraph.

    Defaults: 512^2 circular pupil, 34 x 34 actuators at pitch D/34 (crosstalk 0.15), the actuators with at
    least 10% of their power inside the pupil, nvec = 64 command vectors of N(0, act_rms) (meters at
    lambda0 = 1 m units, i.e. 1e-3 lambda0), FPM radius 4 lambda/D on a q=8, num_airy=32 grid (512^2), Lyot
    stop 0.9 D, final grid q=4, num_airy=32 (256^2); the loss is the intensity summed over the half annulus
    3-12 lambda/D with x > 0.
    """
    from .deformable_mirror import make_gaussian_influence_functions, find_illuminated_actuators
    pupil = make_pupil_grid(pupil_n, 1)
    aperture = circular_aperture(pupil, 1.0)
    inf = make_gaussian_influence_functions(pupil, n_act, 1.0 / n_act, crosstalk=crosstalk)
    inf = find_illuminated_actuators(inf, aperture, 0.1)
    rng = np.random.default_rng(seed)
    actuators = rng.standard_normal((nvec, inf.num_modes)) * act_rms
    fpm_grid = make_focal_grid(fpm_q, fpm_num_airy)
    fpm = 1 - circular_aperture(fpm_grid, 2 * occulter_radius)
    stop = circular_aperture(pupil, stop_diameter)
    focal = make_focal_grid(final_q, final_num_airy)
    x, y = focal.points_list()
    r = np.hypot(x, y)
    roi_mask = (r >= roi[0]) & (r <= roi[1]) & (x > 0)
    return dict(pupil=pupil, aperture=aperture, influence=inf, actuators=actuators, fpm_grid=fpm_grid, fpm=fpm,
                stop=stop, focal=focal, roi=roi_mask)
