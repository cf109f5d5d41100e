"""Fields and mode bases written and read back (hcipy/util/io.py): FITS images with world-coordinate keywords,
npz archives and pickles; the values come back to the device bit for bit."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')
from hcipy_gb300 import io as hio  # noqa: E402


def test_field_round_trips(tmp_path):
    pupil = hg.make_pupil_grid(24, 1.2)
    rng = np.random.default_rng(2)
    real = hg.Field(rng.standard_normal(pupil.size).astype(np.float32), pupil)
    cplx = hg.Field(rng.standard_normal((3, pupil.size)) + 1j * rng.standard_normal((3, pupil.size)), pupil)
    cube = hg.Field(rng.standard_normal((3, pupil.size)), pupil)
    for f, name in ((real, 'r.fits'), (real, 'r.npz'), (real, 'r.pkl'), (cplx, 'c.npz'), (cplx, 'c.pkl'),
                    (cube, 'k.fits')):
        path = str(tmp_path / name)
        hio.write_field(f, path)
        g = hio.read_field(path)
        assert g.data.is_cuda and g.data.dtype == f.data.dtype and g.data.shape == f.data.shape
        assert torch.equal(g.data, f.data)
        assert g.grid.coords.key() == pupil.coords.key()
    with pytest.raises(TypeError):
        hio.write_field(cplx, str(tmp_path / 'c.fits'))
    # the shaped image is what lands in the primary HDU (x fastest)
    hio.write_field(real, str(tmp_path / 's.fits'))
    img = hio.read_fits(str(tmp_path / 's.fits'))
    assert img.shape == (24, 24)
    np.testing.assert_array_equal(img, real.data.cpu().numpy().reshape(24, 24))


def test_reads_a_reference_style_fits_field(tmp_path):
    """The reference's FITS field: primary image, linear WCS keywords (crpix 1, cdelt delta, crval zero) and a
    binary table holding its ASDF tree, which this reader skips."""
    grid = hg.make_pupil_grid(8, 2.0)
    vals = np.arange(64, dtype=np.float64).reshape(8, 8)
    cards = [hio._card('WCSAXES', 2)]
    for i in range(2):
        cards += [hio._card('CRPIX%d' % (i + 1), 1.0), hio._card('CDELT%d' % (i + 1), float(grid.delta[i])),
                  hio._card('CUNIT%d' % (i + 1), ''), hio._card('CTYPE%d' % (i + 1), 'XY'[i]),
                  hio._card('CRVAL%d' % (i + 1), float(grid.zero[i]))]
    table = [hio._card('XTENSION', 'BINTABLE'), hio._card('BITPIX', 8), hio._card('NAXIS', 2),
             hio._card('NAXIS1', 10), hio._card('NAXIS2', 1), hio._card('PCOUNT', 0), hio._card('GCOUNT', 1),
             hio._card('TFIELDS', 1), hio._card('TFORM1', '10B'), hio._card('TTYPE1', 'ASDF_METADATA'),
             hio._card('EXTNAME', 'ASDF'), hio._card('END')]
    path = str(tmp_path / 'ref.fits')
    with open(path, 'wb') as fh:
        fh.write(hio._image_hdu(vals, True, cards) + hio._pad(''.join(table).encode('ascii'), b' ')
                 + hio._pad(b'#ASDF 1.0.', b'\0'))
    f = hio.read_field(path)
    np.testing.assert_array_equal(f.data.cpu().numpy(), vals.ravel())
    np.testing.assert_allclose(f.grid.delta, grid.delta, rtol=1e-15)
    np.testing.assert_allclose(f.grid.zero, grid.zero, rtol=1e-15)
    np.testing.assert_array_equal(f.grid.dims, grid.dims)


def test_mode_basis_round_trips(tmp_path):
    pupil = hg.make_pupil_grid(32, 1)
    basis = hg.make_gaussian_influence_functions(pupil, 6, 1 / 6)
    dense = basis.transformation_matrix.toarray()
    for name in ('b.npz', 'b.pkl', 'b.fits'):
        path = str(tmp_path / name)
        hio.write_mode_basis(basis, path)
        b = hio.read_mode_basis(path)
        m = b.transformation_matrix
        np.testing.assert_array_equal(m.toarray() if hasattr(m, 'toarray') else m, dense)
        assert b.grid.coords.key() == pupil.coords.key()
    # a basis read back drives a deformable mirror like the original
    dm_a, dm_b = hg.DeformableMirror(basis), hg.DeformableMirror(hio.read_mode_basis(str(tmp_path / 'b.pkl')))
    act = np.random.default_rng(3).standard_normal(basis.num_modes) * 1e-3
    dm_a.actuators = act
    dm_b.actuators = act
    assert torch.equal(dm_a.surface.data, dm_b.surface.data)


def test_reads_fields_the_reference_pickled(tmp_path):
    """Fields pickled by the reference's write_field (hcipy/util/io.py:262-266, 316-318): a complex field on a
    regular grid and a real tensor field on a separated grid come back on the device, values bit for bit."""
    from conftest import load_golden
    g = load_golden('io_pickle')
    f = tmp_path / 'reg.pkl'
    f.write_bytes(g['reg_pickle'].tobytes())
    field = hio.read_field(str(f))
    assert isinstance(field, hg.Field) and field.data.is_cuda
    np.testing.assert_array_equal(field.numpy(), g['reg_values'])
    assert field.grid.is_regular
    np.testing.assert_array_equal(np.asarray(field.grid.delta), g['reg_delta'])
    np.testing.assert_array_equal(np.asarray(field.grid.dims), g['reg_dims'])
    np.testing.assert_array_equal(np.asarray(field.grid.zero), g['reg_zero'])
    f = tmp_path / 'sep.pkl'
    f.write_bytes(g['sep_pickle'].tobytes())
    field = hio.read_field(str(f))
    assert field.shape == g['sep_values'].shape
    np.testing.assert_array_equal(field.numpy(), g['sep_values'])
    assert field.grid.is_separated and not field.grid.is_regular
    np.testing.assert_array_equal(np.asarray(field.grid.separated_coords[0]), g['sep_x'])
    np.testing.assert_array_equal(np.asarray(field.grid.separated_coords[1]), g['sep_y'])
