"""FITS, npz and pickle I/O of arrays and grids on the CPU (hcipy/util/io.py).

There is no astropy here to cross-check against, so the FITS files are checked against the standard itself
(FITS 4.0): 2880-byte blocks, fixed-format 80-character cards (value indicator in columns 9-10, logical and
numeric values right-justified to column 30), big-endian data with NAXIS1 the fastest axis, BZERO for unsigned
integers, and extensions of other kinds skipped by their size.
"""
import numpy as np
import pytest

from hcipy_gb300 import io as hio
from hcipy_gb300.field import CartesianGrid, RegularCoords, SeparatedCoords, UnstructuredCoords, make_pupil_grid


@pytest.mark.parametrize('dtype', [np.uint8, np.int8, np.int16, np.uint16, np.int32, np.uint32, np.int64,
                                   np.uint64, np.float32, np.float64, np.bool_])
def test_fits_round_trip(tmp_path, dtype):
    rng = np.random.default_rng(1)
    if dtype == np.bool_:
        a = rng.random((3, 5, 7)) > 0.5
    elif np.issubdtype(dtype, np.integer):
        info = np.iinfo(dtype)
        a = rng.integers(info.min, info.max, size=(3, 5, 7), dtype=dtype, endpoint=True)
        a.flat[0], a.flat[1] = info.min, info.max
    else:
        a = rng.standard_normal((3, 5, 7)).astype(dtype)
    f = str(tmp_path / 'a.fits')
    hio.write_fits(a, f)
    raw = open(f, 'rb').read()
    assert len(raw) % 2880 == 0
    b = hio.read_fits(f)
    assert b.shape == a.shape
    np.testing.assert_array_equal(b, a.astype(np.uint8) if dtype == np.bool_ else a)
    assert b.dtype == (np.uint8 if dtype == np.bool_ else np.dtype(dtype))


def test_fits_layout_follows_the_standard(tmp_path):
    a = np.arange(6, dtype=np.int16).reshape(2, 3)
    f = str(tmp_path / 'a.fits')
    hio.write_fits(a, f)
    raw = open(f, 'rb').read()
    cards = [raw[i:i + 80].decode('ascii') for i in range(0, 2880, 80)]
    assert cards[0][:10] == 'SIMPLE  = ' and cards[0][29] == 'T'
    assert cards[1][:10] == 'BITPIX  = ' and cards[1][10:30].strip() == '16' and cards[1][29] == '6'
    assert cards[2][:10] == 'NAXIS   = ' and cards[2][29] == '2'
    assert cards[3].startswith('NAXIS1  = ') and cards[3][29] == '3'  # the fastest (x) axis first
    assert cards[4].startswith('NAXIS2  = ') and cards[4][29] == '2'
    end = [i for i, c in enumerate(cards) if c.rstrip() == 'END']
    assert len(end) == 1 and all(c == ' ' * 80 for c in cards[end[0] + 1:])
    data = raw[2880:]
    assert len(data) == 2880
    assert data[:12] == a.astype('>i2').tobytes() and data[12:] == b'\0' * (2880 - 12)


def test_fits_unsigned_uses_bzero(tmp_path):
    f = str(tmp_path / 'u.fits')
    hio.write_fits(np.array([0, 1, 65535], np.uint16), f)
    raw = open(f, 'rb').read()
    header = raw[:2880].decode('ascii')
    assert 'BZERO   =                32768' in header and 'BITPIX  =                   16' in header
    assert raw[2880:2886] == np.array([-32768, -32767, 32767], '>i2').tobytes()


def test_fits_skips_other_extensions(tmp_path):
    """A primary image, a binary table (as the reference appends its ASDF tree) and an image extension."""
    img = np.arange(12, dtype=np.float64).reshape(3, 4)
    ext = np.arange(5, dtype=np.int32)
    primary = hio._image_hdu(img, True)
    cards = [hio._card('XTENSION', 'BINTABLE'), hio._card('BITPIX', 8), hio._card('NAXIS', 2),
             hio._card('NAXIS1', 7), hio._card('NAXIS2', 3), hio._card('PCOUNT', 0), hio._card('GCOUNT', 1),
             hio._card('TFIELDS', 1), hio._card('TFORM1', '7B'), hio._card('EXTNAME', 'ASDF'), hio._card('END')]
    table = hio._pad(''.join(cards).encode('ascii'), b' ') + hio._pad(bytes(range(21)), b'\0')
    f = str(tmp_path / 'multi.fits')
    with open(f, 'wb') as fh:
        fh.write(primary + table + hio._image_hdu(ext, False))
    np.testing.assert_array_equal(hio.read_fits(f), img)
    np.testing.assert_array_equal(hio.read_fits(f, 2), ext)
    with pytest.raises(IndexError):
        hio.read_fits(f, 1)


def test_fits_rejects_complex_and_respects_overwrite(tmp_path):
    f = str(tmp_path / 'c.fits')
    with pytest.raises(TypeError):
        hio.write_fits(np.ones(4, np.complex64), f)
    hio.write_fits(np.ones(4), f)
    with pytest.raises(OSError):
        hio.write_fits(np.ones(4), f, overwrite=False)


@pytest.mark.parametrize('ext', ['npz', 'pkl', 'fits'])
def test_grid_round_trip(tmp_path, ext):
    grids = [make_pupil_grid(16, 1.5), CartesianGrid(RegularCoords([0.1, 0.2], [4, 3], [-1.0, 2.0]))]
    if ext != 'fits':
        grids += [CartesianGrid(SeparatedCoords([np.linspace(0, 1, 5), np.geomspace(1, 2, 3)])),
                  CartesianGrid(UnstructuredCoords([np.arange(4.0), np.ones(4)]), weights=np.arange(4.0))]
    for i, g in enumerate(grids):
        f = str(tmp_path / ('g%d.%s' % (i, ext)))
        hio.write_grid(g, f)
        h = hio.read_grid(f)
        assert h.coords.key() == g.coords.key()
        np.testing.assert_allclose(np.broadcast_to(h.weights, (g.size,)), np.broadcast_to(g.weights, (g.size,)))


def test_formats_and_errors(tmp_path):
    g = make_pupil_grid(8)
    with pytest.raises(ValueError):
        hio.write_grid(g, str(tmp_path / 'noext'))
    with pytest.raises(NotImplementedError):
        hio.write_grid(g, str(tmp_path / 'g.asdf'))
    with pytest.raises(NotImplementedError):
        hio.write_grid(CartesianGrid(SeparatedCoords([np.arange(3.0), np.arange(2.0)])), str(tmp_path / 'g.fits'))
    hio.write_grid(g, str(tmp_path / 'g.dat'), fmt='npz')
    assert hio.read_grid(str(tmp_path / 'g.dat'), fmt='npz').coords.key() == g.coords.key()


def test_fits_long_headers_and_scaled_data(tmp_path):
    """Headers longer than one 2880-byte block, long free-format float values, and BSCALE/BZERO scaling of
    integer data (FITS 4.0, section 5.2.5) on reading."""
    data = np.arange(12, dtype=np.int16).reshape(3, 4)
    cards = [hio._card('KEY%d' % i, float(-1.2345678901234567e-05 * (i + 1))) for i in range(60)]
    cards += [hio._card('NOTE', "it's a test"), hio._card('BSCALE', 0.5), hio._card('BZERO', 10.0)]
    raw = hio._image_hdu(data, True, cards)
    f = str(tmp_path / 'scaled.fits')
    with open(f, 'wb') as fh:
        fh.write(raw)
    hdus = hio._read_hdus(open(f, 'rb').read())
    header, got = hdus[0]
    assert len(hdus) == 1
    assert header['NOTE'] == "it's a test"
    np.testing.assert_allclose(header['KEY59'], -1.2345678901234567e-05 * 60, rtol=1e-15)
    np.testing.assert_array_equal(got, data * 0.5 + 10.0)
    assert (len(raw) - 2880) % 2880 == 0 and len(raw) > 2 * 2880  # the header took two blocks


def test_reads_a_grid_the_reference_pickled(tmp_path):
    """An unstructured grid with weights, pickled by the reference's write_grid (hcipy/util/io.py:204-215), reads
    back into this package's grid without the reference installed."""
    from conftest import load_golden
    g = load_golden('io_pickle')
    f = tmp_path / 'grid.pkl'
    f.write_bytes(g['uns_pickle'].tobytes())
    grid = hio.read_grid(str(f))
    assert isinstance(grid, CartesianGrid) and grid.is_unstructured
    np.testing.assert_array_equal(np.asarray(grid.points_list()), g['uns_points'])
    np.testing.assert_array_equal(np.asarray(grid.weights), g['uns_weights'])


def test_reference_pickles_name_only_known_classes(tmp_path):
    """A pickle that names another class of the reference is refused instead of importing anything."""
    import pickle
    f = tmp_path / 'other.pkl'
    f.write_bytes(b'chcipy.optics\nWavefront\n.')  # protocol 0: GLOBAL hcipy.optics.Wavefront, STOP
    with pytest.raises(pickle.UnpicklingError, match='not a reference field or grid class'):
        hio.read_grid(str(f))
