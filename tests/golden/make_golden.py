"""Generate the golden vectors in this folder by running the HCIPy reference itself.

The reference is pure Python; it imports here through the small stand-ins in
``refshim/`` (numexpr -> numpy eval, numba -> identity decorators, xxhash ->
blake2b, a minimal YAML reader, numpy-only array_api_compat, and import stubs
for the plotting / FITS packages that the diffraction path never calls).

Usage (from the repository root, with the reference checked out read-only)::

    python tests/golden/make_golden.py REFERENCE_SOURCE_TREE [case ...]

REFERENCE_SOURCE_TREE is the directory that holds the reference's ``hcipy``
package (required).  With case names (the ``make_<case>`` functions below,
e.g. ``pickle_case``) only those cases are regenerated.

Every case is small and seeded; the outputs are written as compressed ``.npz``
files next to this script.  Nothing in the test suite runs this script: the
tests only read the ``.npz`` files, so they run where the reference is absent.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(path):
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(HERE, 'refshim'))
    sys.path.insert(0, path)
    import packaging.version  # noqa: F401  (the reference's io module needs it pre-imported)
    import hcipy
    return hcipy


def grid_record(prefix, grid):
    """Store the regular-grid description (delta, dims, zero) of a grid."""
    return {
        prefix + '_delta': np.asarray(grid.delta, dtype=np.float64),
        prefix + '_dims': np.asarray(grid.dims, dtype=np.int64),
        prefix + '_zero': np.asarray(grid.zero, dtype=np.float64),
        prefix + '_weights': np.asarray(np.broadcast_to(grid.weights, (grid.size,)), dtype=np.float64),
    }


def separated_record(prefix, grid):
    x, y = grid.separated_coords
    return {prefix + '_x': np.asarray(x, np.float64), prefix + '_y': np.asarray(y, np.float64)}


def random_field(rng, grid, aperture=None):
    e = rng.standard_normal(grid.size) + 1j * rng.standard_normal(grid.size)
    if aperture is not None:
        e = e * aperture
    return e


def make_mft_cases(hp, out):
    rng = np.random.default_rng(11)
    cases = [
        # (pupil dims, pupil diameter, focal q, num_airy, scale)
        ((64, 64), 1.0, 4, 8, 2 * np.pi),
        ((48, 40), 1.3, 3, (5, 7), 2 * np.pi / 1.7),
        ((33, 31), 0.8, 2.5, 6.3, 2 * np.pi * 1.1),
    ]
    for i, (dims, diam, q, num_airy, scale) in enumerate(cases):
        pupil = hp.make_pupil_grid(dims, diam)
        focal = hp.make_focal_grid(q, num_airy).scaled(scale).shifted([0.013 * i, -0.02 * i])
        e = random_field(rng, pupil)
        f = random_field(rng, focal)
        mft = hp.MatrixFourierTransform(pupil, focal)
        rec = {}
        rec.update(separated_record('in', pupil))
        rec.update(separated_record('out', focal))
        rec.update(grid_record('ingrid', pupil))
        rec.update(grid_record('outgrid', focal))
        rec['E'] = e
        rec['F'] = f
        rec['fwd_c128'] = np.asarray(mft.forward(hp.Field(e, pupil)))
        rec['bwd_c128'] = np.asarray(mft.backward(hp.Field(f, focal)))
        rec['fwd_c64'] = np.asarray(mft.forward(hp.Field(e.astype(np.complex64), pupil)))
        rec['bwd_c64'] = np.asarray(mft.backward(hp.Field(f.astype(np.complex64), focal)))
        out['mft_%d' % i] = rec

    # One-dimensional MFT.
    g1 = hp.make_uniform_grid(37, 1.0)
    f1 = hp.make_uniform_grid(29, 40.0, center=0.3)
    mft1 = hp.MatrixFourierTransform(g1, f1)
    e = random_field(rng, g1)
    f = random_field(rng, f1)
    out['mft_1d'] = {
        'in_x': np.asarray(g1.x, np.float64), 'out_x': np.asarray(f1.x, np.float64),
        'w_in': np.float64(g1.weights), 'w_out': np.float64(f1.weights),
        'E': e, 'F': f,
        'fwd_c128': np.asarray(mft1.forward(hp.Field(e, g1))),
        'bwd_c128': np.asarray(mft1.backward(hp.Field(f, f1))),
    }


def make_fraunhofer_cfg1(hp, out):
    """The 256^2 circular pupil with a 0.1 rad RMS Zernike 2-21 phase to a 128^2 focal grid."""
    pupil = hp.make_pupil_grid(256, 1)
    aperture = hp.make_circular_aperture(1)(pupil)
    zb = hp.make_zernike_basis(20, 1, pupil, starting_mode=2)
    rng = np.random.default_rng(0)
    c = rng.standard_normal(20)
    phase = zb.linear_combination(c)
    inside = aperture > 0
    phase = phase * (0.1 / np.std(phase[inside]))
    e = aperture * np.exp(1j * phase)
    focal = hp.make_focal_grid(q=4, num_airy=16)
    prop = hp.FraunhoferPropagator(pupil, focal)
    wf = hp.Wavefront(hp.Field(e, pupil), 1)
    res128 = prop.forward(wf).electric_field
    wf64 = hp.Wavefront(hp.Field(e.astype(np.complex64), pupil), 1)
    res64 = prop.forward(wf64).electric_field
    back = prop.backward(hp.Wavefront(res128, 1)).electric_field
    out['fraunhofer_cfg1'] = {
        'E': e.astype(np.complex128), 'focal_c128': np.asarray(res128), 'focal_c64': np.asarray(res64),
        'back_c128': np.asarray(back),
        **grid_record('pupil', pupil), **grid_record('focal', focal),
    }


def make_fft_cases(hp, out):
    rng = np.random.default_rng(22)
    cases = [
        ((32, 32), 1.0, 2, 1, 0),
        ((15, 17), 0.7, 3, 0.75, (0.5, -1.2)),
        ((16, 12), 2.0, 1.5, 0.8, 0.3),
        ((20, 20), 1.0, 1, 1, 0),
    ]
    for i, (dims, diam, q, fov, shift) in enumerate(cases):
        pupil = hp.make_pupil_grid(dims, diam)
        fft = hp.FastFourierTransform(pupil, q=q, fov=fov, shift=shift)
        fft2 = hp.FastFourierTransform(pupil, q=q, fov=fov, shift=shift, emulate_fftshifts=False)
        e = random_field(rng, pupil)
        f = random_field(rng, fft.output_grid)
        out['fft_%d' % i] = {
            'q': np.float64(q), 'fov': np.float64(fov), 'shift': np.broadcast_to(np.asarray(shift, np.float64), (2,)).copy(),
            'E': e, 'F': f,
            'fwd_c128': np.asarray(fft.forward(hp.Field(e, pupil))),
            'bwd_c128': np.asarray(fft.backward(hp.Field(f, fft.output_grid))),
            'fwd_exact_c128': np.asarray(fft2.forward(hp.Field(e, pupil))),
            'fwd_c64': np.asarray(fft.forward(hp.Field(e.astype(np.complex64), pupil))),
            **grid_record('ingrid', pupil), **grid_record('outgrid', fft.output_grid),
            **grid_record('internal', fft.internal_grid),
        }


def make_czt_cases(hp, out):
    rng = np.random.default_rng(33)
    recs = {}
    for i, (n, m) in enumerate([(37, 23), (64, 100), (101, 7), (250, 250)]):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        w = np.exp(1j * rng.uniform(0, 2 * np.pi))
        a = np.exp(1j * rng.uniform(0, 2 * np.pi))
        czt = hp.ChirpZTransform(n, m, w, a)
        recs['x_%d' % i] = x
        recs['w_%d' % i] = np.complex128(w)
        recs['a_%d' % i] = np.complex128(a)
        recs['y_%d' % i] = np.asarray(czt(x))
        recs['y64_%d' % i] = np.asarray(czt(x.astype(np.complex64)))
        recs['n_%d' % i] = np.int64(n)
        recs['m_%d' % i] = np.int64(m)
    # A batched call along the last axis.
    xb = rng.standard_normal((3, 5, 19)) + 1j * rng.standard_normal((3, 5, 19))
    czt = hp.ChirpZTransform(19, 31, np.exp(-0.2j), np.exp(0.7j))
    recs['xb'] = xb
    recs['yb'] = np.asarray(czt(xb))
    out['czt'] = recs

    # ZoomFFT on a small grid.
    pupil = hp.make_pupil_grid((24, 20), 1)
    focal = hp.make_focal_grid(3, (5, 4)).scaled(2 * np.pi).shifted([0.1, -0.2])
    zfft = hp.ZoomFastFourierTransform(pupil, focal)
    e = random_field(rng, pupil)
    f = random_field(rng, focal)
    out['zoomfft'] = {
        'E': e, 'F': f,
        'fwd_c128': np.asarray(zfft.forward(hp.Field(e, pupil))),
        'bwd_c128': np.asarray(zfft.backward(hp.Field(f, focal))),
        **grid_record('ingrid', pupil), **grid_record('outgrid', focal),
    }


def make_asp_cases(hp, out):
    rng = np.random.default_rng(44)
    recs = {}
    # The native transfer-function branch (large distance relative to sampling is the other branch).
    for i, (n, diam, wl, d) in enumerate([(64, 8.0, 1.6e-6, 0.5), (48, 8.0, 1.6e-6, 5.0), (40, 2e-3, 500e-9, 0.05),
                                          (32, 1e-3, 1e-6, 1.0)]):
        pupil = hp.make_pupil_grid(n, diam)
        aperture = hp.make_circular_aperture(diam * 0.9)(pupil)
        e = aperture * np.exp(1j * rng.standard_normal(pupil.size) * 0.3)
        asp = hp.AngularSpectrumPropagator(pupil, d)
        wf = hp.Wavefront(hp.Field(e, pupil), wl)
        fwd = asp.forward(wf).electric_field
        bwd = asp.backward(hp.Wavefront(fwd, wl)).electric_field
        fwd64 = asp.forward(hp.Wavefront(hp.Field(e.astype(np.complex64), pupil), wl)).electric_field
        # Which branch did the reference take?
        L_max = np.max(np.asarray(pupil.dims) * pupil.delta)
        impulse_branch = bool(np.any(pupil.delta < wl * abs(d) / L_max))
        recs['case_%d' % i] = {
            'n': np.int64(n), 'diam': np.float64(diam), 'wavelength': np.float64(wl), 'distance': np.float64(d),
            'E': e, 'fwd_c128': np.asarray(fwd), 'bwd_c128': np.asarray(bwd), 'fwd_c64': np.asarray(fwd64),
            'impulse_branch': np.bool_(impulse_branch),
        }
    out.update({'asp_%d' % i: r for i, r in enumerate(recs.values())})

    # FourierFilter with a generic scalar transfer function, q=2.
    g = hp.make_pupil_grid((30, 26), 1.0)
    def tf(fg):
        return hp.Field(np.exp(-0.01 * (fg.x**2 + 2 * fg.y**2)) * np.exp(0.3j * fg.x), fg)
    ff = hp.FourierFilter(g, tf, q=2)
    e = random_field(rng, g)
    internal = ff.internal_grid
    out['fourier_filter'] = {
        'E': e, 'fwd_c128': np.asarray(ff.forward(hp.Field(e, g))), 'bwd_c128': np.asarray(ff.backward(hp.Field(e, g))),
        'tf': np.asarray(tf(internal)),
        **grid_record('ingrid', g), **grid_record('internal', internal),
    }


def make_fresnel_cases(hp, out):
    """FresnelPropagator (hcipy/propagation/fresnel.py) in both branches, two zero paddings, two media."""
    rng = np.random.default_rng(45)
    cases = [(64, 8.0, 1.6e-6, 0.5, 2, 1.0), (48, 8.0, 1.6e-6, 5000.0, 2, 1.0), (40, 2e-3, 500e-9, 0.05, 3, 1.0),
             (32, 1e-3, 1e-6, 1.0, 2, 1.0), (36, 1e-3, 1e-6, 0.3, 2, 1.5)]
    for i, (n, diam, wl, d, q, nref) in enumerate(cases):
        pupil = hp.make_pupil_grid(n, diam)
        aperture = hp.make_circular_aperture(diam * 0.9)(pupil)
        e = aperture * np.exp(1j * rng.standard_normal(pupil.size) * 0.3)
        prop = hp.FresnelPropagator(pupil, d, zero_padding=q, refractive_index=nref)
        wf = hp.Wavefront(hp.Field(e, pupil), wl)
        fwd = prop.forward(wf).electric_field
        bwd = prop.backward(hp.Wavefront(fwd, wl)).electric_field
        L_max = np.max(np.asarray(pupil.dims) * pupil.delta)
        out['fresnel_%d' % i] = {
            'n': np.int64(n), 'diam': np.float64(diam), 'wavelength': np.float64(wl), 'distance': np.float64(d),
            'zero_padding': np.int64(q), 'refractive_index': np.float64(nref),
            'E': e, 'fwd_c128': np.asarray(fwd), 'bwd_c128': np.asarray(bwd),
            'impulse_branch': np.bool_(bool(np.any(pupil.delta < wl * abs(d) / L_max))),
        }


def make_vortex_cases(hp, out):
    """VortexCoronagraph (hcipy/coronagraphy/vortex.py:12-15 on multi_scale.py:10-161): charge 2 and 4, the
    Lyot-plane field of an aberrated circular pupil, and the backward propagation of a random Lyot-plane field."""
    rng = np.random.default_rng(46)
    for i, (n, charge, q, sf, ws) in enumerate([(64, 2, 64, 4, 32), (48, 4, 32, 2, 16)]):
        pupil = hp.make_pupil_grid(n, 1.0)
        aperture = hp.make_circular_aperture(1.0)(pupil)
        e = aperture * np.exp(1j * 0.05 * rng.standard_normal(pupil.size))
        vortex = hp.VortexCoronagraph(pupil, charge, q=q, scaling_factor=sf, window_size=ws)
        lyot = vortex.forward(hp.Wavefront(hp.Field(e, pupil), 1.0)).electric_field
        g = random_field(rng, pupil)
        back = vortex.backward(hp.Wavefront(hp.Field(g, pupil), 1.0)).electric_field
        rec = {'n': np.int64(n), 'charge': np.int64(charge), 'q': np.int64(q), 'scaling_factor': np.int64(sf),
               'window_size': np.int64(ws), 'E': e, 'lyot_c128': np.asarray(lyot), 'G': g,
               'back_c128': np.asarray(back), 'levels': np.int64(len(vortex.focal_masks))}
        for k, m in enumerate(vortex.focal_masks):
            rec['mask_%d' % k] = np.asarray(m)
        out['vortex_%d' % i] = rec


def make_vector_vortex_case(hp, out):
    """VectorVortexCoronagraph (hcipy/coronagraphy/vortex.py:17-246), charge 2 on a 48^2 pupil (q 32, scaling
    factor 2, window 16, a Lyot stop, a retardance that depends on the wavelength): the Lyot-plane Jones matrix of
    an unpolarised aberrated pupil at two wavelengths and the Stokes parameters of its image (the polarised
    wavefront's I/Q/U/V, hcipy/optics/wavefront.py:103-255); a partially polarised input; the backward propagation
    of a random Jones-matrix field and of a scalar field."""
    rng = np.random.default_rng(49)
    pupil = hp.make_pupil_grid(48, 1.0)
    aperture = hp.make_circular_aperture(1.0)(pupil)
    stop = hp.make_circular_aperture(0.9)(pupil)
    e = aperture * np.exp(1j * 0.05 * rng.standard_normal(pupil.size))
    vvc = hp.VectorVortexCoronagraph(2, lyot_stop=stop, phase_retardation=lambda wl: np.pi * (1 + 0.05 * (wl - 1)),
                                     q=32, scaling_factor=2, window_size=16)
    prop = hp.FraunhoferPropagator(pupil, hp.make_focal_grid(4, 8))
    rec = {'E': e, 'stop': np.asarray(stop)}
    for k, wl in enumerate((1.0, 1.1)):
        lyot = vvc.forward(hp.Wavefront(hp.Field(e, pupil), wl))
        rec['lyot_%d' % k] = np.asarray(lyot.electric_field)
        rec['lyot_stokes_%d' % k] = np.asarray(lyot.input_stokes_vector, np.float64)
        img = prop(lyot)
        rec['image_%d' % k] = np.stack([np.asarray(img.I), np.asarray(img.Q), np.asarray(img.U), np.asarray(img.V)])
        rec['wavelength_%d' % k] = np.float64(wl)
    ej = (rng.standard_normal((2, 2, pupil.size)) + 1j * rng.standard_normal((2, 2, pupil.size))) * aperture
    stokes = np.array([1.0, 0.3, -0.2, 0.1])
    lyot = vvc.forward(hp.Wavefront(hp.Field(ej, pupil), 1.0, stokes))
    rec.update({'EJ': ej, 'stokes': stokes, 'lyot_pol': np.asarray(lyot.electric_field),
                'lyot_pol_stokes': np.asarray(lyot.stokes_vector)})
    g = rng.standard_normal((2, 2, pupil.size)) + 1j * rng.standard_normal((2, 2, pupil.size))
    rec['G'] = g
    rec['back'] = np.asarray(vvc.backward(hp.Wavefront(hp.Field(g, pupil), 1.0, stokes)).electric_field)
    rec['back_scalar'] = np.asarray(vvc.backward(hp.Wavefront(hp.Field(g[0, 0], pupil), 1.0)).electric_field)
    out['vector_vortex'] = rec


def make_planner_case(hp, out):
    """The method choice of make_fourier_transform(planner='estimate') (hcipy/fourier/fourier_transform.py:217-300)
    over pupils of 16^2 to 2048^2 and rectangular ones, FFT output grids of q 1-16 and fov 1-0.1 and focal grids
    that are not FFT grids: for every case the expected time of each supported method (the reference's operation
    counts and time model) and the method it picks, taken from the reference's own classes."""
    from hcipy.fourier.fast_fourier_transform import FastFourierTransform
    from hcipy.fourier.matrix_fourier_transform import MatrixFourierTransform
    from hcipy.fourier.naive_fourier_transform import NaiveFourierTransform
    from hcipy.fourier.zoom_fast_fourier_transform import ZoomFastFourierTransform
    methods = [('fft', FastFourierTransform), ('mft', MatrixFourierTransform), ('naive', NaiveFourierTransform),
               ('zft', ZoomFastFourierTransform)]
    rec = {'methods': np.array([m for m, _ in methods])}
    cases = []
    for dims, diam in [(16, 1.0), (32, 1.0), (64, 2.0), (100, 1.0), (128, 1.0), (256, 1.0), (512, 8.0), (1024, 8.0),
                       (2048, 1.0), ((96, 64), (1.5, 1.0)), ((33, 47), 1.0)]:
        for q in (1, 2, 4, 8, 16):
            for fov in (1, 0.5, 0.25, 0.1):
                cases.append((dims, diam, q, fov, None))
        for q, num_airy in ((2, 8), (4, 16), (8, 32), (3.3, 12.5)):
            cases.append((dims, diam, q, num_airy, 'focal'))
    inputs, params, kinds, times, best = [], [], [], [], []
    for dims, diam, q, x, kind in cases:
        pupil = hp.make_pupil_grid(dims, diam)
        if kind is None:
            output_grid = hp.make_fft_grid(pupil, q, x)
            allowed = [m for m, _ in methods]
        else:
            # a focal grid in angular-frequency units, as FraunhoferPropagator builds it (not an FFT grid)
            output_grid = hp.make_focal_grid(q, x, spatial_resolution=1.0).scaled(2 * np.pi / np.max(
                np.asarray(pupil.delta) * np.asarray(pupil.dims)))
            allowed = [m for m, _ in methods]
            try:
                hp.fourier.fast_fourier_transform.get_fft_parameters(output_grid, pupil)
            except ValueError:
                allowed.remove('fft')
        t = []
        for m, cls in methods:
            if m in allowed and cls.is_supported(pupil, output_grid):
                t.append(cls.compute_complexity(pupil, output_grid).expected_execution_time)
            else:
                t.append(np.nan)
        inputs.append(np.broadcast_to(np.asarray(dims, np.int64), (2,)))
        params.append([np.max(np.broadcast_to(np.asarray(diam, np.float64), (2,))) if kind else 0.0, q, x,
                       1.0 if kind else 0.0])
        kinds.append(np.broadcast_to(np.asarray(diam, np.float64), (2,)))
        times.append(t)
        best.append(int(np.nanargmin(t)))
    rec.update({'dims': np.array(inputs), 'diameter': np.array(kinds), 'params': np.array(params),
                'times': np.array(times), 'best': np.array(best)})
    out['planner'] = rec


def make_fft_grid_case(hp, out):
    """FFT-grid algebra (hcipy/fourier/fast_fourier_transform.py:23-154) over square, rectangular and odd pupils with
    q, fov and shift varied: the output grid of make_fft_grid and what get_fft_parameters recovers from it."""
    rows = []
    for dims, diam in [(16, 1.0), (33, 1.0), (64, 2.0), (100, 1.3), ((96, 64), (1.5, 1.0)), ((31, 48), (0.7, 1.1))]:
        pupil = hp.make_pupil_grid(dims, diam)
        for q in (1, 1.5, 2, 4, 8):
            for fov in (1, 0.5, 0.3):
                for shift in (0, 0.25, (0.5, -1.2)):
                    g = hp.make_fft_grid(pupil, q, fov, shift)
                    qq, ff, ss = hp.fourier.fast_fourier_transform.get_fft_parameters(g, pupil)
                    b = lambda v: np.broadcast_to(np.asarray(v, np.float64), (2,))  # noqa: E731
                    rows.append(np.concatenate([b(dims), b(diam), [q, fov], b(shift), b(g.delta), b(g.dims),
                                                b(g.zero), b(qq), b(ff), b(ss)]))
    out['fft_grids'] = {'rows': np.array(rows),
                        'columns': np.array(['dims', 'diameter', 'q', 'fov', 'shift', 'delta', 'out_dims', 'zero',
                                             'q_found', 'fov_found', 'shift_found'])}


def make_host_functions_case(hp, out):
    """Host helpers with the reference's outputs: make_uniform_grid (odd and even sizes, centres, has_center),
    make_pupil_grid, make_focal_grid (spatial resolution, pupil diameter + focal length + wavelength, f-number),
    make_focal_grid_from_pupil_grid,
    the Cn^2 / Fried-parameter conversions and the von Karman covariance and PSD
    (hcipy/field/util.py:68-318, hcipy/atmosphere/atmospheric_model.py:321-399)."""
    grids = []

    def row(g):
        """ndim, then delta, dims and zero per axis, padded to two axes with NaN."""
        vals = [np.asarray(v, np.float64).ravel() for v in (g.delta, g.dims, g.zero)]
        pad = [np.concatenate([v, np.full(2 - len(v), np.nan)]) for v in vals]
        return np.concatenate([[len(vals[0])]] + pad)

    for dims, extent, center, has_center in [(8, 1.0, 0, False), (9, 1.0, 0, False), (9, 2.0, 0, True),
                                             (10, 2.0, 0, True), ((6, 7), (1.0, 1.4), (0.1, -0.3), False),
                                             ((6, 7), (1.0, 1.4), (0.1, -0.3), True)]:
        g = hp.make_uniform_grid(dims, extent, center, has_center)
        grids.append(row(g))
    for dims, diam in [(64, 1.0), (65, 2.0), ((40, 30), (1.0, 0.75))]:
        g = hp.make_pupil_grid(dims, diam)
        grids.append(row(g))
    for kw in [dict(q=4, num_airy=16), dict(q=3.3, num_airy=(8, 5.5)), dict(q=2, num_airy=10, spatial_resolution=0.5),
               dict(q=4, num_airy=8, pupil_diameter=8.0, focal_length=20.0, reference_wavelength=1.6e-6),
               dict(q=5, num_airy=6, f_number=12.0, reference_wavelength=7e-7)]:
        g = hp.make_focal_grid(**kw)
        grids.append(row(g))
    for dims, diam, kw in [(64, 1.0, dict(q=4, num_airy=16)),
                           ((40, 30), (1.0, 0.75), dict(q=3, num_airy=(8, 6), focal_length=2.0, wavelength=0.5)),
                           (33, 2.0, dict(q=2))]:
        grids.append(row(hp.make_focal_grid_from_pupil_grid(hp.make_pupil_grid(dims, diam), **kw)))
    r0s = np.array([0.05, 0.1, 0.15, 0.3])
    wls = np.array([500e-9, 1.6e-6])
    cn2 = np.array([[hp.Cn_squared_from_fried_parameter(r, wl) for r in r0s] for wl in wls])
    back = np.array([[hp.fried_parameter_from_Cn_squared(c, wl) for c in row] for row, wl in zip(cn2, wls)])
    fg = hp.make_pupil_grid(24, 40.0)
    psd = np.asarray(hp.power_spectral_density_von_karman(0.12, 22.0)(fg))
    r = np.array([0.0, 1e-3, 0.05, 0.3, 1.0, 4.0, 25.0])
    from hcipy.atmosphere.atmospheric_model import phase_covariance_von_karman
    cov = np.asarray(phase_covariance_von_karman(0.12, 22.0)(hp.CartesianGrid(hp.UnstructuredCoords((r, 0 * r)))))
    out['host_functions'] = {'grids': np.array(grids), 'r0': r0s, 'wavelengths': wls, 'cn2': cn2,
                             'r0_back': back, 'psd': psd, 'cov_r': r, 'cov': cov}


def make_influence_sweep_case(hp, out):
    """Gaussian influence functions (hcipy/optics/deformable_mirror.py:43-93) beyond the default: other crosstalk
    and cutoff values, x/y/z tilts of the mirror and oversampled evaluation, on a 24^2 pupil with 5 x 5
    actuators; each basis stored as its CSR arrays."""
    pupil = hp.make_pupil_grid(24, 1.0)
    rec = {}
    cases = [dict(crosstalk=0.15, cutoff=3), dict(crosstalk=0.3, cutoff=2), dict(crosstalk=0.15, cutoff=3, x_tilt=0.1),
             dict(crosstalk=0.15, cutoff=3, y_tilt=0.2, z_tilt=0.3), dict(crosstalk=0.2, cutoff=2.5, oversampling=2),
             dict(crosstalk=0.15, cutoff=3, z_tilt=0.25, oversampling=3)]
    for i, kw in enumerate(cases):
        basis = hp.make_gaussian_influence_functions(pupil, 5, 1 / 5, **kw)
        import scipy.sparse
        m = scipy.sparse.csr_matrix(basis.transformation_matrix)
        m.sort_indices()
        rec['data_%d' % i], rec['indices_%d' % i], rec['indptr_%d' % i] = m.data, m.indices, m.indptr
        rec['shape_%d' % i] = np.array(m.shape)
        for k in ('crosstalk', 'cutoff', 'x_tilt', 'y_tilt', 'z_tilt', 'oversampling'):
            rec['%s_%d' % (k, i)] = np.float64(kw.get(k, {'oversampling': 1}.get(k, 0.0)))
    rec['count'] = np.int64(len(cases))
    out['influence_sweep'] = rec


def make_atmosphere_matrices_case(hp, out):
    """InfiniteAtmosphericLayer's stencils and autoregressive matrices (infinite_atmospheric_layer.py:111-202) for
    a rectangular grid, a longer stencil and another outer scale and seed."""
    rec = {}
    for i, (dims, diam, stencil_length, L0, seed) in enumerate([((20, 14), (1.0, 0.7), 2, 25.0, 11),  # noqa: N806
                                                                (16, 2.0, 3, 8.0, 12)]):
        pupil = hp.make_pupil_grid(dims, diam)
        layer = hp.InfiniteAtmosphericLayer(pupil, hp.Cn_squared_from_fried_parameter(0.2, 500e-9), L0=L0,
                                            stencil_length=stencil_length, seed=seed)
        rec.update({'A_vertical_%d' % i: layer.A_vertical, 'B_vertical_%d' % i: layer.B_vertical,
                    'A_horizontal_%d' % i: layer.A_horizontal, 'B_horizontal_%d' % i: layer.B_horizontal,
                    'stencil_bottom_%d' % i: layer.stencil_bottom_idx.astype(np.int64),
                    'stencil_left_%d' % i: layer.stencil_left_idx.astype(np.int64),
                    'dims_%d' % i: np.asarray(pupil.dims, np.int64), 'delta_%d' % i: np.asarray(pupil.delta),
                    'zero_%d' % i: np.asarray(pupil.zero), 'stencil_length_%d' % i: np.int64(stencil_length),
                    'L0_%d' % i: np.float64(L0), 'seed_%d' % i: np.int64(seed)})
    rec['count'] = np.int64(2)
    out['atmosphere_matrices'] = rec


def make_pyramid_case(hp, out):
    """PyramidWavefrontSensorOptics (hcipy/wavefront_sensing/pyramid.py:94-199): forward of an aberrated pupil at
    two wavelengths (the pyramid phase depends on the refractive index and the wavenumber), backward of a random
    field on the sensor's pupil plane."""
    rng = np.random.default_rng(47)
    pupil = hp.make_pupil_grid(48, 1.0)
    wfs_grid = hp.make_pupil_grid(96, 2.0)
    pwfs = hp.PyramidWavefrontSensorOptics(pupil, wfs_grid, separation=1.0, pupil_diameter=1.0, wavelength_0=1.0,
                                           refractive_index=lambda wl: 1.5 + 0.01 * (wl - 1.0))
    aperture = hp.make_circular_aperture(1.0)(pupil)
    e = aperture * np.exp(0.2j * rng.standard_normal(pupil.size))
    rec = {'E': e, 'G': random_field(rng, wfs_grid)}
    for k, wl in enumerate((1.0, 1.2)):
        rec['fwd_%d' % k] = np.asarray(pwfs.forward(hp.Wavefront(hp.Field(e, pupil), wl)).electric_field)
        rec['wavelength_%d' % k] = np.float64(wl)
    rec['bwd'] = np.asarray(pwfs.backward(hp.Wavefront(hp.Field(rec['G'], wfs_grid), 1.0)).electric_field)
    rec.update(grid_record('focal', pwfs.focal_grid))
    out['pyramid'] = rec


def make_modulated_pyramid_case(hp, out):
    """ModulatedPyramidWavefrontSensorOptics (hcipy/wavefront_sensing/pyramid.py:10-91): 6 modulation steps of
    radius 3 lambda/D, the tip-tilt form at one wavelength and the shifted-pyramid form at two; TipTiltMirror
    (hcipy/optics/tip_tilt_mirror.py) alone for one command."""
    rng = np.random.default_rng(53)
    pupil = hp.make_pupil_grid(32, 1.0)
    wfs_grid = hp.make_pupil_grid(40, 2.0)
    pwfs = hp.PyramidWavefrontSensorOptics(pupil, wfs_grid, separation=1.0, pupil_diameter=1.0, wavelength_0=1.0,
                                           refractive_index=lambda wl: 1.5 + 0.01 * (wl - 1.0))
    aperture = hp.make_circular_aperture(1.0)(pupil)
    e = aperture * np.exp(0.2j * rng.standard_normal(pupil.size))
    rec = {'E': e, 'modulation': np.float64(3.0), 'num_steps': np.int64(6)}
    slow = hp.ModulatedPyramidWavefrontSensorOptics(pwfs, 3.0, num_steps=6)
    rec['positions'] = np.asarray(slow.modulation_positions.points)
    rec['slow'] = np.stack([np.asarray(w.electric_field) for w in slow.forward(hp.Wavefront(hp.Field(e, pupil), 1.0))])
    fast = hp.ModulatedPyramidWavefrontSensorOptics(pwfs, 3.0, num_steps=6, fast_modulation_method=True)
    for k, wl in enumerate((1.0, 1.2)):
        wfs = fast.forward(hp.Wavefront(hp.Field(e, pupil), wl))
        rec['fast_%d' % k] = np.stack([np.asarray(w.electric_field) for w in wfs])
        rec['wavelength_%d' % k] = np.float64(wl)
    rec['fast_surface_3'] = np.asarray(fast._pyramid_apodizers[3].surface_sag)
    ttm = hp.TipTiltMirror(pupil)
    ttm.actuators = np.array([2e-3, -1e-3])
    rec['tip_tilt_command'] = np.asarray(ttm.actuators)
    rec['tip_tilt'] = np.asarray(ttm.forward(hp.Wavefront(hp.Field(e, pupil), 0.8)).electric_field)
    out['modulated_pyramid'] = rec


def make_lyot_case(hp, out):
    """A 128^2 pupil Lyot chain: focal-plane mask radius 4 lambda/D on a q=8 num_airy=8 grid."""
    pupil = hp.make_pupil_grid(128, 1)
    aperture = hp.make_circular_aperture(1)(pupil)
    zb = hp.make_zernike_basis(30, 1, pupil, starting_mode=2)
    rng = np.random.default_rng(3)
    c = rng.standard_normal(30)
    phase = zb.linear_combination(c)
    phase *= 2 * np.pi * 1e-2 / np.std(phase[aperture > 0])
    e = aperture * np.exp(1j * phase)
    fpm_grid = hp.make_focal_grid(8, 8)
    fpm = 1 - hp.make_circular_aperture(8)(fpm_grid)
    stop = hp.make_circular_aperture(0.9)(pupil)
    lyot = hp.LyotCoronagraph(pupil, fpm, stop)
    focal = hp.make_focal_grid(4, 16)
    prop = hp.FraunhoferPropagator(pupil, focal)
    wf = hp.Wavefront(hp.Field(e, pupil), 1)
    lyot_plane = lyot.forward(wf).electric_field
    img = prop.forward(hp.Wavefront(lyot_plane, 1)).electric_field
    ref_img = prop.forward(hp.Wavefront(hp.Field(aperture.astype(complex), pupil), 1)).power
    wf64 = hp.Wavefront(hp.Field(e.astype(np.complex64), pupil), 1)
    lyot64 = lyot.forward(wf64).electric_field
    out['lyot'] = {
        'E': e, 'aperture': np.asarray(aperture), 'fpm': np.asarray(fpm), 'stop': np.asarray(stop),
        'lyot_c128': np.asarray(lyot_plane), 'lyot_c64': np.asarray(lyot64), 'image_c128': np.asarray(img),
        'ref_peak': np.float64(np.max(ref_img)),
        **grid_record('pupil', pupil), **grid_record('fpm', fpm_grid), **grid_record('focal', focal),
    }


def make_subpixel_cases(hp, out):
    from hcipy._math import subpixel_shift as sp
    rng = np.random.default_rng(55)
    img = rng.standard_normal((40, 50))
    recs = {'img': img}
    shifts = [(0.3, -0.2), (-0.5, 0.5), (0.0, 0.11), (-0.37, 0.0)]
    for i, (dy, dx) in enumerate(shifts):
        recs['dy_%d' % i] = np.float64(dy)
        recs['dx_%d' % i] = np.float64(dx)
        recs['out_%d' % i] = sp.subpixel_shift(img, dy, dx)
        recs['wy_%d' % i] = sp._quintic_weights(dy)
        recs['wx_%d' % i] = sp._quintic_weights(dx)
    out['subpixel'] = recs


def make_atmosphere_case(hp, out):
    """InfiniteAtmosphericLayer on a 24^2 grid: matrices, stencils and an extrusion replay."""
    import copy
    pupil = hp.make_pupil_grid(24, 1.0)
    cn2 = hp.Cn_squared_from_fried_parameter(0.2, 500e-9)
    layer = hp.InfiniteAtmosphericLayer(pupil, cn2, L0=25, velocity=(3.0, 0.0), use_interpolation=True, seed=5)
    rec = {
        'A_vertical': layer.A_vertical, 'B_vertical': layer.B_vertical,
        'A_horizontal': layer.A_horizontal, 'B_horizontal': layer.B_horizontal,
        'stencil_bottom_idx': layer.stencil_bottom_idx.astype(np.int64),
        'stencil_left_idx': layer.stencil_left_idx.astype(np.int64),
        'screen0': np.asarray(layer._achromatic_screen), 'cn2': np.float64(cn2),
        'cov_vertical': layer.cov_matrix_vertical,
    }
    # Replay: record the noise of each extrusion by drawing from a copy of the generator.
    noises = []
    screens = []
    kinds = []
    dts = [0.011, 0.013, 0.004]
    t = 0.0
    for dt in dts:
        rng_copy = copy.deepcopy(layer.rng)
        old = np.round(layer.center / pupil.delta).astype('int')
        new_center = layer.center + layer.velocity * dt
        new = np.round(new_center / pupil.delta).astype('int')
        nsteps = int(abs(new[0] - old[0]))
        noise = [rng_copy.normal(0, np.sqrt(cn2), size=layer.B_horizontal.shape[1]) for _ in range(nsteps)]
        t += dt
        layer.t = t
        noises.append(np.array(noise).reshape((nsteps, layer.B_horizontal.shape[1])))
        screens.append(np.asarray(layer._achromatic_screen))
        kinds.append(np.asarray(layer.phase_for(1.0)))
    for i in range(len(dts)):
        rec['noise_%d' % i] = noises[i]
        rec['screen_%d' % i] = screens[i]
        rec['shifted_%d' % i] = kinds[i]
        rec['dt_%d' % i] = np.float64(dts[i])
    rec['velocity'] = np.asarray(layer.velocity, dtype=np.float64)
    rec.update(grid_record('pupil', pupil))
    out['atmosphere'] = rec


def make_dm_case(hp, out):
    pupil = hp.make_pupil_grid(64, 1)
    inf = hp.make_gaussian_influence_functions(pupil, 8, 1 / 8, crosstalk=0.15)
    dm = hp.DeformableMirror(inf)
    rng = np.random.default_rng(66)
    dm.actuators = rng.standard_normal(dm.num_actuators) * 1e-3
    e = hp.make_circular_aperture(1)(pupil).astype(complex)
    wf = hp.Wavefront(hp.Field(e, pupil), 1.0)
    out['dm'] = {
        'influence': np.asarray(inf.transformation_matrix.toarray() if hasattr(inf.transformation_matrix, 'toarray') else inf.transformation_matrix),
        'actuators': dm.actuators.copy(), 'surface': np.asarray(dm.surface),
        'E': e, 'fwd_c128': np.asarray(dm.forward(wf).electric_field),
        **grid_record('pupil', pupil),
    }


def make_efc_case(hp, out):
    """Electric-field conjugation on a 32^2 pupil: a 6x6 Gaussian DM, the Lyot coronagraph (radius 2 lambda/D
    mask) and the lens onto a 32^2 image; the tutorial's poke Jacobian over a one-sided dark zone (2.5-7 lambda/D,
    x > 0.5), its Tikhonov inverse (hcipy.inverse_tikhonov), five EFC iterations against a seeded aberration; and
    the three regularised inverses (hcipy/util/matrix_inversion.py) of a seeded ill-conditioned matrix."""
    rng = np.random.default_rng(48)
    pupil = hp.make_pupil_grid(32, 1)
    aperture = hp.make_circular_aperture(1)(pupil)
    inf = hp.make_gaussian_influence_functions(pupil, 6, 1 / 6, crosstalk=0.15)
    dm = hp.DeformableMirror(inf)
    fpm_grid = hp.make_focal_grid(8, 6)
    fpm = 1 - hp.make_circular_aperture(4)(fpm_grid)
    stop = hp.make_circular_aperture(0.9)(pupil)
    lyot = hp.LyotCoronagraph(pupil, fpm, stop)
    focal = hp.make_focal_grid(2, 8)
    prop = hp.FraunhoferPropagator(pupil, focal)
    r = np.hypot(focal.x, focal.y)
    dark_zone = (r >= 2.5) & (r <= 7) & (focal.x > 0.5)
    aberration = np.exp(1j * 0.02 * rng.standard_normal(pupil.size)) * aperture
    epsilon, rcond, gain = 1e-3, 1e-2, 0.5

    def get_field(actuators, aberrated):
        dm.actuators = actuators
        e = aberration if aberrated else aperture.astype(complex)
        return np.asarray(prop(lyot(dm(hp.Wavefront(hp.Field(e, pupil), 1.0)))).electric_field)

    # the tutorial's poke Jacobian (E(+eps) - E(-eps)) eps / var(+-eps), written out for this case
    amps = np.linspace(-epsilon, epsilon, 2)
    cols = []
    for i in range(dm.num_actuators):
        resp = sum(a * get_field(a * np.eye(dm.num_actuators)[i], False) for a in amps) / np.var(amps)
        cols.append(np.concatenate((resp[dark_zone].real, resp[dark_zone].imag)))
    jac = np.array(cols).T
    efc_matrix = hp.inverse_tikhonov(jac, rcond)
    act = np.zeros(dm.num_actuators)
    history, dz_ni = [], []
    peak = np.abs(np.asarray(prop(hp.Wavefront(hp.Field(aperture.astype(complex), pupil), 1.0)).electric_field)).max()**2
    for _ in range(5):
        e = get_field(act, True)
        history.append(act.copy())
        dz_ni.append(np.mean(np.abs(e[dark_zone])**2) / peak)
        x = np.concatenate((e[dark_zone].real, e[dark_zone].imag))
        act = act - gain * efc_matrix.dot(x)
    m = rng.standard_normal((40, 12)) @ np.diag(np.logspace(0, -6, 12)) @ rng.standard_normal((12, 12))
    out['efc'] = {
        'influence': np.asarray(inf.transformation_matrix.toarray()), 'aperture': np.asarray(aperture),
        'aberration': np.asarray(aberration), 'fpm': np.asarray(fpm), 'stop': np.asarray(stop),
        'dark_zone': np.asarray(dark_zone), 'epsilon': np.float64(epsilon), 'rcond': np.float64(rcond),
        'gain': np.float64(gain), 'jacobian': jac, 'efc_matrix': efc_matrix, 'actuators': np.array(history),
        'dark_zone_ni': np.array(dz_ni), 'peak': np.float64(peak),
        'M': m, 'M_tikhonov': hp.inverse_tikhonov(m, 1e-3), 'M_truncated': hp.inverse_truncated(m, 1e-4),
        'M_modal': hp.inverse_truncated_modal(m, 5),
        **grid_record('pupil', pupil), **grid_record('fpm', fpm_grid), **grid_record('focal', focal),
    }


def make_pickle_case(hp, out):
    """Fields and grids pickled by the reference's own writers (hcipy/util/io.py:204-215, 262-266, 296-320): a
    complex field on a regular grid, a real tensor field on a separated grid and an unstructured grid with
    weights, each as the bytes of the file the reference wrote, with the values and grids they hold."""
    import pickle
    import tempfile
    rng = np.random.default_rng(21)
    reg = hp.make_pupil_grid([12, 10], [1.2, 1.0])
    f_reg = hp.Field(rng.standard_normal(reg.size) + 1j * rng.standard_normal(reg.size), reg)
    sep = hp.CartesianGrid(hp.SeparatedCoords([np.sort(rng.uniform(-1, 1, 7)), np.sort(rng.uniform(-2, 2, 5))]))
    f_sep = hp.Field(rng.standard_normal((3, sep.size)), sep)
    pts = rng.standard_normal((2, 9))
    uns = hp.CartesianGrid(hp.UnstructuredCoords(pts), rng.uniform(0.5, 1.5, 9))
    rec = {'reg_values': np.asarray(f_reg), 'reg_delta': np.asarray(reg.delta, np.float64),
           'reg_dims': np.asarray(reg.dims, np.int64), 'reg_zero': np.asarray(reg.zero, np.float64),
           'sep_values': np.asarray(f_sep), 'sep_x': np.asarray(sep.separated_coords[0]),
           'sep_y': np.asarray(sep.separated_coords[1]), 'uns_points': pts,
           'uns_weights': np.asarray(uns.weights, np.float64)}
    with tempfile.TemporaryDirectory() as d:
        for name, obj, writer in [('reg', f_reg, hp.write_field), ('sep', f_sep, hp.write_field),
                                  ('uns', uns, hp.write_grid)]:
            path = os.path.join(d, name + '.pkl')
            writer(obj, path, fmt='pickle')
            with open(path, 'rb') as f:
                rec[name + '_pickle'] = np.frombuffer(f.read(), np.uint8)
            with open(path, 'rb') as f:
                pickle.load(f)  # the reference reads its own file back
    out['io_pickle'] = rec


def make_spectral_noise_case(hp, out):
    """Multi-scale spectral noise (hcipy/util/spectral_noise.py:203-320) with the von Karman PSD
    (hcipy/atmosphere/atmospheric_model.py:376-399) on a rectangular grid: the screen of one seeded realization,
    and the same realization shifted."""
    grid = hp.make_pupil_grid([40, 32], [2.0, 1.6])
    r0, L0 = 0.15, 12.0  # noqa: N806
    psd = hp.power_spectral_density_von_karman(r0, L0)
    factory = hp.SpectralNoiseFactoryMultiscale(psd, grid, 4)
    noise = factory.make_random(9)
    shift = np.array([0.13, -0.07])
    out['spectral_noise'] = {
        'screen': np.asarray(noise()), 'shifted': np.asarray(noise.shifted(shift)()), 'shift': shift,
        'r0': np.float64(r0), 'L0': np.float64(L0), 'oversampling': np.int64(4), 'seed': np.int64(9),
        **grid_record('grid', grid),
    }


def save(out):
    for name, rec in out.items():
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)
        print('wrote', name, sum(np.asarray(v).nbytes for v in rec.values()), 'bytes')


CASES = ['mft_cases', 'fraunhofer_cfg1', 'fft_cases', 'czt_cases', 'asp_cases', 'fresnel_cases', 'vortex_cases',
         'vector_vortex_case', 'planner_case', 'fft_grid_case', 'host_functions_case',
         'influence_sweep_case', 'atmosphere_matrices_case',
         'pyramid_case', 'modulated_pyramid_case', 'lyot_case', 'subpixel_cases',
         'atmosphere_case', 'dm_case', 'efc_case', 'pickle_case', 'spectral_noise_case']


def main():
    if len(sys.argv) < 2:
        sys.exit('usage: make_golden.py REFERENCE_SOURCE_TREE [case ...]  (cases: %s)' % ' '.join(CASES))
    hp = import_reference(sys.argv[1])
    chosen = sys.argv[2:] or CASES
    unknown = [c for c in chosen if c not in CASES]
    if unknown:
        sys.exit('unknown case(s): %s' % ' '.join(unknown))
    out = {}
    for case in chosen:
        globals()['make_' + case](hp, out)
    save(out)


if __name__ == '__main__':
    main()
