"""Reading and writing arrays, grids, fields and mode bases (hcipy/util/io.py:38-430).

Formats, picked from the file name as the reference does (``_guess_file_format``, io.py:86-106) or by ``fmt``:

* ``fits``: the FITS standard (version 4.0) written and read here without astropy.  ``write_fits``/``read_fits``
  hold plain real arrays (ints, floats, booleans as bytes).  A field goes into the primary image, grid axes
  unflattened, with the linear world-coordinate keywords the reference writes beside it (CRPIX = 1, CDELT =
  delta, CRVAL = zero, CTYPE = X/Y/...), so a regular grid comes back from the header; the reference's own
  FITS field files (primary image + the same keywords + an ASDF table, which is skipped) read back the same
  way.  A mode basis is a cube (modes, y, x) with the same keywords.  FITS has no complex images: complex
  data raise ``TypeError`` (the reference's astropy path rejects them too); use ``npz``.
* ``npz``: numpy archive with the values and the grid's description (regular, separated or unstructured
  coordinates and weights); complex data welcome.
* ``pickle``: Python pickles of this package's objects, with the device tensors moved to host memory.  Pickles
  that the reference wrote (its fields, old- and new-style, and its Cartesian grids with regular, separated or
  unstructured coordinates) read back too, into this package's objects, without the reference installed.
* ``asdf``: not built (the asdf package is not part of this build): ``NotImplementedError``.

Data read back land on the device as the other operators expect.
"""
import os
import pickle

import numpy as np
import scipy.sparse

from .field import CartesianGrid, RegularCoords, SeparatedCoords, UnstructuredCoords, Field

_BLOCK = 2880
_CARD = 80
_BITPIX = {np.dtype(np.uint8): 8, np.dtype('>i2'): 16, np.dtype('>i4'): 32, np.dtype('>i8'): 64,
           np.dtype('>f4'): -32, np.dtype('>f8'): -64}
_FROM_BITPIX = {8: np.dtype(np.uint8), 16: np.dtype('>i2'), 32: np.dtype('>i4'), 64: np.dtype('>i8'),
                -32: np.dtype('>f4'), -64: np.dtype('>f8')}


# ---------------------------------------------------------------------------
# FITS cards and HDUs
# ---------------------------------------------------------------------------

def _card(key, value=None, comment=None):
    """One 80-character header card in the fixed format (FITS 4.0, section 4.2)."""
    key = key.upper()
    if len(key) > 8:
        raise ValueError('FITS keyword longer than 8 characters: %r' % key)
    if value is None:
        s = key.ljust(8)
    else:
        if isinstance(value, (bool, np.bool_)):
            v = ('T' if value else 'F').rjust(20)
        elif isinstance(value, (int, np.integer)):
            v = str(int(value)).rjust(20)
        elif isinstance(value, (float, np.floating)):
            v = repr(float(value)).upper()
            if 'E' not in v and '.' not in v and v not in ('NAN', 'INF', '-INF'):
                v += '.'
            v = v.rjust(20)
        else:
            text = str(value).replace("'", "''")
            v = ("'" + text.ljust(8) + "'").ljust(20)
        s = key.ljust(8) + '= ' + v
        if comment:
            s += ' / ' + comment
    if len(s) > _CARD:
        raise ValueError('FITS card too long: %r' % s)
    return s.ljust(_CARD)


def _pad(b, fill):
    r = len(b) % _BLOCK
    return b if r == 0 else b + fill * (_BLOCK - r)


def _image_hdu(data, primary, extra_cards=()):
    """Header and data bytes of one image HDU for a real numpy array (``None``: no data)."""
    cards = [_card('SIMPLE', True)] if primary else [_card('XTENSION', 'IMAGE')]
    bzero = None
    if data is None:
        cards += [_card('BITPIX', 8), _card('NAXIS', 0)]
        raw = b''
    else:
        a = np.asarray(data)
        if np.iscomplexobj(a):
            raise TypeError('FITS images hold real values only; write complex data with fmt="npz".')
        if a.dtype == np.bool_:
            a = a.astype(np.uint8)
        elif a.dtype.kind == 'u' and a.dtype.itemsize > 1:
            # unsigned integers: the signed type with BZERO = 2^(bits-1) (FITS 4.0, section 5.2.5); flipping the
            # top bit is the subtraction of 2^(bits-1) in two's complement
            bits = 8 * a.dtype.itemsize
            bzero = 1 << (bits - 1)
            a = (a.astype(a.dtype.newbyteorder('=')) ^ a.dtype.type(bzero)).view('i%d' % a.dtype.itemsize)
            a = a.astype(a.dtype.newbyteorder('>'))
        elif a.dtype == np.int8:
            bzero = -128
            a = (a.astype(np.int16) + 128).astype(np.uint8)
        elif a.dtype.kind in 'iuf':
            a = a.astype(a.dtype.newbyteorder('>'))
        else:
            raise TypeError('no FITS image type for %s' % a.dtype)
        if a.dtype.kind == 'f' and a.dtype.itemsize == 2:
            a = a.astype('>f4')
        bitpix = _BITPIX[np.dtype(a.dtype)]
        cards += [_card('BITPIX', bitpix), _card('NAXIS', a.ndim)]
        cards += [_card('NAXIS%d' % (i + 1), n) for i, n in enumerate(a.shape[::-1])]
        raw = np.ascontiguousarray(a).tobytes()
    if primary:
        cards.append(_card('EXTEND', True))
    else:
        cards += [_card('PCOUNT', 0), _card('GCOUNT', 1)]
    if bzero is not None:
        cards += [_card('BSCALE', 1), _card('BZERO', bzero)]
    cards += list(extra_cards)
    cards.append(_card('END'))
    header = _pad(''.join(cards).encode('ascii'), b' ')
    return header + _pad(raw, b'\0')


def _parse_value(text):
    text = text.strip()
    if text.startswith("'"):
        end = 1
        out = []
        while end < len(text):
            ch = text[end]
            if ch == "'":
                if end + 1 < len(text) and text[end + 1] == "'":
                    out.append("'")
                    end += 2
                    continue
                break
            out.append(ch)
            end += 1
        return ''.join(out).rstrip()
    text = text.split('/')[0].strip()
    if text == 'T':
        return True
    if text == 'F':
        return False
    try:
        return int(text)
    except ValueError:
        pass
    try:
        return float(text.replace('D', 'E'))
    except ValueError:
        return text


def _read_hdus(buf):
    """[(header dict, data array or None)] of every HDU in the bytes of a FITS file."""
    pos, hdus = 0, []
    while pos + _BLOCK <= len(buf):
        header, ended = {}, False
        while not ended:
            if pos + _BLOCK > len(buf):
                raise ValueError('truncated FITS header')
            block = buf[pos:pos + _BLOCK].decode('ascii')
            pos += _BLOCK
            for i in range(0, _BLOCK, _CARD):
                card = block[i:i + _CARD]
                key = card[:8].strip()
                if key == 'END':
                    ended = True
                    break
                if card[8:10] == '= ' and key:
                    header[key] = _parse_value(card[10:])
        if not hdus and header.get('SIMPLE') is not True:
            raise ValueError('not a FITS file (no SIMPLE = T)')
        bitpix, naxis = int(header['BITPIX']), int(header['NAXIS'])
        dims = [int(header['NAXIS%d' % (i + 1)]) for i in range(naxis)]
        count = int(np.prod(dims)) if naxis else 0
        size = abs(bitpix) // 8 * int(header.get('GCOUNT', 1)) * (int(header.get('PCOUNT', 0)) + count)
        data = None
        is_image = not hdus or header.get('XTENSION', '').strip() == 'IMAGE'
        if is_image and count:
            data = np.frombuffer(buf, dtype=_FROM_BITPIX[bitpix], count=count, offset=pos).reshape(dims[::-1])
            bscale, bzero = header.get('BSCALE', 1), header.get('BZERO', 0)
            if bitpix == 8 and bzero == -128 and bscale == 1:
                data = (data.astype(np.int16) - 128).astype(np.int8)
            elif bitpix > 8 and bscale == 1 and bzero == 1 << (bitpix - 1):
                u = np.dtype('u%d' % (bitpix // 8))
                data = data.astype(data.dtype.newbyteorder('=')).view(u) ^ u.type(bzero)
            elif bscale != 1 or bzero != 0:
                data = data * bscale + bzero
            else:
                data = data.astype(data.dtype.newbyteorder('='))
        pos += (size + _BLOCK - 1) // _BLOCK * _BLOCK
        hdus.append((header, data))
    return hdus


def _write_bytes(filename, payload, overwrite):
    if os.path.exists(filename) and not overwrite:
        raise OSError('File %r already exists.' % filename)
    with open(filename, 'wb') as f:
        f.write(payload)


def _host(x):
    if isinstance(x, Field):
        x = x.data
    if hasattr(x, 'detach'):
        x = x.detach().cpu().numpy()
    return np.asarray(x)


def read_fits(filename, extension=0):
    """The data of HDU ``extension`` of a FITS file (io.py:38-53)."""
    with open(filename, 'rb') as f:
        hdus = _read_hdus(f.read())
    data = hdus[extension][1]
    if data is None:
        raise IndexError('No data in HDU #%d.' % extension)
    return data.copy()


def write_fits(data, filename, shape=None, overwrite=True):
    """An array or Field as the primary image of a FITS file (io.py:55-84); a Field on a separated grid is
    written with its grid axes unflattened, ``shape`` overrides that."""
    arr = _host(data)
    if shape is not None:
        arr = arr.reshape(shape)
    elif isinstance(data, Field) and data.grid is not None and data.grid.is_separated:
        arr = arr.reshape(arr.shape[:-1] + data.grid.shape)
    _write_bytes(filename, _image_hdu(arr, True), overwrite)


# ---------------------------------------------------------------------------
# Grids
# ---------------------------------------------------------------------------

def _guess_file_format(filename):
    if filename.endswith('asdf'):
        return 'asdf'
    if filename.endswith('fits') or filename.endswith('fits.gz'):
        return 'fits'
    if filename.endswith('pkl') or filename.endswith('pickle'):
        return 'pickle'
    if filename.endswith('npz'):
        return 'npz'
    return None


def _format(filename, fmt):
    if fmt is None:
        fmt = _guess_file_format(filename)
        if fmt is None:
            raise ValueError('Format not given and could not be guessed based on the file extension.')
    if fmt == 'asdf':
        raise NotImplementedError('The "asdf" file format needs the asdf package, which this build does not use.')
    if fmt not in ('fits', 'pickle', 'npz'):
        raise NotImplementedError('The "%s" file format has not been implemented.' % fmt)
    if fmt == 'fits' and filename.endswith('.gz'):
        raise NotImplementedError('Compressed FITS files are not supported.')
    return fmt


def _grid_arrays(grid, prefix='grid_'):
    c = grid.coords
    out = {}
    if c.is_regular:
        out.update({prefix + 'type': np.array('regular'), prefix + 'delta': np.asarray(c.delta, np.float64),
                    prefix + 'dims': np.asarray(c.dims, np.int64), prefix + 'zero': np.asarray(c.zero, np.float64)})
    elif c.is_separated:
        out[prefix + 'type'] = np.array('separated')
        for i, s in enumerate(c.separated_coords):
            out[prefix + 'coord%d' % i] = np.asarray(s, np.float64)
    else:
        out[prefix + 'type'] = np.array('unstructured')
        for i, v in enumerate(c.flat()):
            out[prefix + 'coord%d' % i] = np.asarray(v, np.float64)
    if grid._weights is not None:
        out[prefix + 'weights'] = np.asarray(np.broadcast_to(grid._weights, ()) if np.ndim(grid._weights) == 0
                                             else grid._weights, np.float64)
    return out


def _grid_from_arrays(d, prefix='grid_'):
    kind = str(d[prefix + 'type'])
    if kind == 'regular':
        coords = RegularCoords(d[prefix + 'delta'], d[prefix + 'dims'], d[prefix + 'zero'])
    else:
        n = sum(1 for k in d if k.startswith(prefix + 'coord'))
        arrs = [np.asarray(d[prefix + 'coord%d' % i]) for i in range(n)]
        coords = SeparatedCoords(arrs) if kind == 'separated' else UnstructuredCoords(arrs)
    w = d.get(prefix + 'weights')
    if w is not None:
        w = np.asarray(w)
        w = float(w) if w.ndim == 0 else w
    return CartesianGrid(coords, w)


# ---- pickles written by the reference ---------------------------------------------------------------------
#
# The reference pickles its Field either as an ndarray subclass (hcipy/field/field.py:113-135, 175-211: the
# ndarray state plus the grid) or as a wrapper whose state is {'data', 'grid'} (:512-541), its CartesianGrid with
# the default instance dict {'coords', '_weights'} (hcipy/field/grid.py:31), and its coordinates with small state
# dicts (hcipy/field/coordinates.py:264-277, 420-433, 623-641).  The unpickler below maps those classes onto
# stand-ins that keep the state, and the stand-ins are converted to this package's grids and fields.

class _RefState(object):
    """Keeps the pickled state of one reference object."""

    def __init__(self, *args):
        self.state = None

    def __setstate__(self, state):
        self.state = state


class _RefOldField(_RefState):
    pass


class _RefNewField(_RefState):
    pass


class _RefGrid(_RefState):
    pass


class _RefRegular(_RefState):
    pass


class _RefSeparated(_RefState):
    pass


class _RefUnstructured(_RefState):
    pass


def _ref_field_reconstruct(subtype, baseclass, baseshape, basetype):
    return subtype()


_REF_CLASSES = {
    ('hcipy.field.field', '_field_reconstruct'): _ref_field_reconstruct,
    ('hcipy.field.field', 'OldStyleField'): _RefOldField,
    ('hcipy.field.field', 'NewStyleField'): _RefNewField,
    ('hcipy.field.field', 'Field'): _RefNewField,
    ('hcipy.field.cartesian_grid', 'CartesianGrid'): _RefGrid,
    ('hcipy.field.coordinates', 'RegularCoords'): _RefRegular,
    ('hcipy.field.coordinates', 'SeparatedCoords'): _RefSeparated,
    ('hcipy.field.coordinates', 'UnstructuredCoords'): _RefUnstructured,
}


class _Unpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module.startswith('hcipy.') or module == 'hcipy':
            cls = _REF_CLASSES.get((module, name))
            if cls is None:
                raise pickle.UnpicklingError('%s.%s: not a reference field or grid class this reader knows'
                                             % (module, name))
            return cls
        return super().find_class(module, name)


def _from_ref(obj):
    """Reference stand-ins -> this package's objects (anything else passes through)."""
    if isinstance(obj, _RefOldField):
        _, shape, dtype, fortran, raw, grid = obj.state
        arr = np.ndarray.__new__(np.ndarray, (0,), 'b')
        arr.__setstate__((shape, dtype, fortran, raw))
        return Field(np.ascontiguousarray(arr), _from_ref(grid))
    if isinstance(obj, _RefNewField):
        return Field(np.ascontiguousarray(np.asarray(obj.state['data'])), _from_ref(obj.state['grid']))
    if isinstance(obj, _RefGrid):
        w = obj.state.get('_weights')
        if w is not None:
            w = np.asarray(w)
            w = float(w) if w.ndim == 0 else w
        return CartesianGrid(_from_ref(obj.state['coords']), w)
    if isinstance(obj, _RefRegular):
        st = obj.state
        return RegularCoords(np.asarray(st['delta'], np.float64), np.asarray(st['dims'], np.int64),
                             np.asarray(st['zero'], np.float64))
    if isinstance(obj, _RefSeparated):
        return SeparatedCoords([np.asarray(c, np.float64) for c in obj.state['separated_coords']])
    if isinstance(obj, _RefUnstructured):
        return UnstructuredCoords([np.asarray(c, np.float64) for c in obj.state['coords']])
    return obj


def _load_pickle(filename):
    with open(filename, 'rb') as f:
        return _from_ref(_Unpickler(f).load())


def _wcs_cards(grid):
    if grid is None or not grid.is_regular:
        return []
    axes = 'XYZW'
    cards = [_card('WCSAXES', grid.ndim)]
    for i in range(grid.ndim):
        cards += [_card('CRPIX%d' % (i + 1), 1.0), _card('CDELT%d' % (i + 1), float(grid.delta[i])),
                  _card('CRVAL%d' % (i + 1), float(grid.zero[i])), _card('CTYPE%d' % (i + 1), axes[i])]
    return cards


def _grid_from_wcs(header, ndim):
    try:
        delta, zero, dims = [], [], []
        for i in range(ndim):
            crpix = float(header['CRPIX%d' % (i + 1)])
            d = float(header['CDELT%d' % (i + 1)])
            delta.append(d)
            zero.append(float(header['CRVAL%d' % (i + 1)]) - (crpix - 1) * d)
            dims.append(int(header['NAXIS%d' % (i + 1)]))
    except KeyError:
        return None
    return CartesianGrid(RegularCoords(delta, dims, zero))


def write_grid(grid, filename, fmt=None, overwrite=True):
    """A grid to a file (io.py:176-215).  FITS holds regular grids only, as header keywords of an empty
    primary HDU (NAXISn then give the dimensions through HXDIMn)."""
    fmt = _format(filename, fmt)
    if fmt == 'pickle':
        return _write_bytes(filename, pickle.dumps(grid), overwrite)
    if fmt == 'npz':
        if os.path.exists(filename) and not overwrite:
            raise OSError('File %r already exists.' % filename)
        with open(filename, 'wb') as f:
            np.savez(f, **_grid_arrays(grid))
        return
    if not grid.is_regular:
        raise NotImplementedError('Only regular grids can be written to FITS here; use fmt="npz".')
    cards = _wcs_cards(grid) + [_card('HXDIM%d' % (i + 1), int(n)) for i, n in enumerate(grid.dims)]
    _write_bytes(filename, _image_hdu(None, True, cards), overwrite)


def read_grid(filename, fmt=None):
    """A grid from a file (io.py:134-174)."""
    fmt = _format(filename, fmt)
    if fmt == 'pickle':
        return _load_pickle(filename)
    if fmt == 'npz':
        with np.load(filename) as d:
            return _grid_from_arrays(dict(d))
    with open(filename, 'rb') as f:
        header = _read_hdus(f.read())[0][0]
    n = int(header.get('WCSAXES', 0))
    if n == 0 or 'HXDIM1' not in header:
        raise ValueError('%r holds no grid description this reader knows.' % filename)
    hdr = dict(header)
    for i in range(n):
        hdr['NAXIS%d' % (i + 1)] = header['HXDIM%d' % (i + 1)]
    return _grid_from_wcs(hdr, n)


# ---------------------------------------------------------------------------
# Fields
# ---------------------------------------------------------------------------

def write_field(field, filename, fmt=None, overwrite=True):
    """A Field to a file (io.py:268-321)."""
    fmt = _format(filename, fmt)
    if fmt == 'pickle':
        return _write_bytes(filename, pickle.dumps(field), overwrite)
    values = _host(field)
    grid = field.grid if isinstance(field, Field) else None
    if fmt == 'npz':
        if os.path.exists(filename) and not overwrite:
            raise OSError('File %r already exists.' % filename)
        arrays = {'values': values}
        if grid is not None:
            arrays.update(_grid_arrays(grid))
        with open(filename, 'wb') as f:
            np.savez(f, **arrays)
        return
    if grid is None or not grid.is_regular:
        raise NotImplementedError('FITS fields need a regular grid here; use fmt="npz".')
    shaped = values.reshape(values.shape[:-1] + grid.shape)
    _write_bytes(filename, _image_hdu(shaped, True, _wcs_cards(grid)), overwrite)


def read_field(filename, fmt=None):
    """A Field from a file (io.py:217-266), on the device."""
    fmt = _format(filename, fmt)
    if fmt == 'pickle':
        return _load_pickle(filename)
    if fmt == 'npz':
        with np.load(filename) as d:
            d = dict(d)
        grid = _grid_from_arrays(d) if 'grid_type' in d else None
        return Field(d['values'], grid)
    with open(filename, 'rb') as f:
        header, data = _read_hdus(f.read())[0]
    if data is None:
        raise ValueError('%r has no primary image.' % filename)
    ndim = int(header.get('WCSAXES', 0)) or data.ndim
    grid = _grid_from_wcs(header, ndim)
    if grid is None:
        raise ValueError('%r has no linear world-coordinate keywords to rebuild the grid from.' % filename)
    return Field(np.ascontiguousarray(data.reshape(data.shape[:data.ndim - ndim] + (-1,))), grid)


# ---------------------------------------------------------------------------
# Mode bases
# ---------------------------------------------------------------------------

def write_mode_basis(mode_basis, filename, fmt=None, overwrite=True):
    """A ModeBasis to a file (io.py:374-430)."""
    fmt = _format(filename, fmt)
    if fmt == 'pickle':
        return _write_bytes(filename, pickle.dumps(mode_basis), overwrite)
    m = mode_basis.transformation_matrix
    grid = mode_basis.grid
    if fmt == 'npz':
        if os.path.exists(filename) and not overwrite:
            raise OSError('File %r already exists.' % filename)
        if scipy.sparse.issparse(m):
            c = scipy.sparse.csr_matrix(m)
            arrays = {'sparse': np.array(True), 'data': c.data, 'indices': c.indices, 'indptr': c.indptr,
                      'shape': np.asarray(c.shape, np.int64)}
        else:
            arrays = {'sparse': np.array(False), 'matrix': np.asarray(m)}
        if grid is not None:
            arrays.update(_grid_arrays(grid))
        with open(filename, 'wb') as f:
            np.savez(f, **arrays)
        return
    if grid is None or not grid.is_regular:
        raise NotImplementedError('FITS mode bases need a regular grid here; use fmt="npz".')
    dense = m.toarray() if scipy.sparse.issparse(m) else np.asarray(m)
    cube = np.ascontiguousarray(dense.T.reshape((-1,) + grid.shape))
    _write_bytes(filename, _image_hdu(cube, True, _wcs_cards(grid)), overwrite)


def read_mode_basis(filename, fmt=None):
    """A ModeBasis from a file (io.py:323-372); FITS cubes come back dense."""
    from .deformable_mirror import ModeBasis
    fmt = _format(filename, fmt)
    if fmt == 'pickle':
        return _load_pickle(filename)
    if fmt == 'npz':
        with np.load(filename) as d:
            d = dict(d)
        grid = _grid_from_arrays(d) if 'grid_type' in d else None
        if bool(d['sparse']):
            m = scipy.sparse.csr_matrix((d['data'], d['indices'], d['indptr']), shape=tuple(d['shape']))
        else:
            m = d['matrix']
        return ModeBasis(m, grid)
    with open(filename, 'rb') as f:
        header, data = _read_hdus(f.read())[0]
    if data is None:
        raise ValueError('%r has no primary image.' % filename)
    ndim = int(header.get('WCSAXES', 0)) or data.ndim - 1
    grid = _grid_from_wcs(header, ndim)
    modes = data.reshape(data.shape[:data.ndim - ndim] + (-1,))
    return ModeBasis(np.ascontiguousarray(modes.reshape(-1, modes.shape[-1]).T), grid)
