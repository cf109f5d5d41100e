"""Element-wise and sparse device operations behind the optical elements (phase screens, influence functions).

Every function launches a kernel of ``lib/libhcipy_gb300.so``; there is no CPU path.
"""
import numpy as np
import torch

from . import _lib

_REAL = {torch.complex64: torch.float32, torch.complex128: torch.float64}


def _batched(t, n):
    """(batch, n) contiguous view of a tensor whose last axis has n elements."""
    t = t.contiguous()
    if t.shape[-1] != n:
        raise ValueError('expected a last axis of %d elements, got %s' % (n, tuple(t.shape)))
    return t.reshape(-1, n)


def apply_phase(e, s, scale):
    """e * exp(i * scale * s) with broadcasting of a leading batch (e or s may hold one field).

    e: complex tensor (..., n); s: real tensor (..., n).  The result has the broader of the two batch shapes and
    e's dtype; s is cast to the matching real type.
    """
    n = e.shape[-1]
    rdt = _REAL[e.dtype]
    s = s.to(device=e.device, dtype=rdt)
    shape_e, shape_s = tuple(e.shape[:-1]), tuple(s.shape[:-1])
    be = int(np.prod(shape_e)) if shape_e else 1
    bs = int(np.prod(shape_s)) if shape_s else 1
    batch = max(be, bs) if be and bs else 0  # an empty batch on either side gives an empty result
    try:
        lead = tuple(torch.broadcast_shapes(shape_e, shape_s))  # keeps a batch of one given on either side
    except RuntimeError:
        lead = shape_e if be >= bs else shape_s
    out_shape = (lead if int(np.prod(lead)) == batch else (shape_e if be >= bs else shape_s)) + (n,)
    e2, s2 = _batched(e, n), _batched(s, n)
    out = torch.empty(out_shape, dtype=e.dtype, device=e.device)
    if out.numel() == 0:
        return out
    rc = _lib.lib().hx_phase_apply(n, batch, be, bs, _lib.dptr(e2), _lib.dtype_code(e.dtype), _lib.dptr(s2),
                                   float(scale), _lib.dptr(out), _lib.stream_handle())
    _lib.check(rc, 'hx_phase_apply')
    return out


def apply_phase_grad(e, s, scale, g_out, need_e=True, need_s=True):
    """Gradients of ``apply_phase`` for real s: (g_e, g_s), each reduced to its input's batch shape."""
    n = e.shape[-1]
    rdt = _REAL[e.dtype]
    s = s.to(device=e.device, dtype=rdt)
    shape_e, shape_s = tuple(e.shape[:-1]), tuple(s.shape[:-1])
    be = int(np.prod(shape_e)) if shape_e else 1
    bs = int(np.prod(shape_s)) if shape_s else 1
    batch = max(be, bs) if be and bs else 0  # an empty batch on either side gives an empty result
    e2, s2 = _batched(e, n), _batched(s, n)
    g2 = _batched(g_out.to(e.dtype), n)
    g_e = torch.empty(shape_e + (n,), dtype=e.dtype, device=e.device) if need_e else None
    g_s = torch.empty(shape_s + (n,), dtype=rdt, device=e.device) if need_s else None
    if batch == 0 or n == 0:  # an empty batch contributes nothing to a shared input's gradient
        return (None if g_e is None else g_e.zero_()), (None if g_s is None else g_s.zero_())
    rc = _lib.lib().hx_phase_apply_grad(n, batch, be, bs, _lib.dptr(e2), _lib.dtype_code(e.dtype), _lib.dptr(s2),
                                        float(scale), _lib.dptr(g2), None if g_s is None else _lib.dptr(g_s),
                                        None if g_e is None else _lib.dptr(g_e), _lib.stream_handle())
    _lib.check(rc, 'hx_phase_apply_grad')
    return g_e, g_s


class SparseBasis(object):
    """A sparse (npix x nact) influence-function matrix on the device, in CSR (pixels) and CSC (actuators) form."""

    def __init__(self, csr, device, dtype):
        import scipy.sparse
        csr = scipy.sparse.csr_matrix(csr)
        csr.sort_indices()
        csc = csr.tocsc()
        csc.sort_indices()
        self.shape = csr.shape
        self.dtype = dtype
        self.row_ptr = torch.from_numpy(csr.indptr.astype(np.int32)).to(device)
        self.col_idx = torch.from_numpy(csr.indices.astype(np.int32)).to(device)
        self.vals = torch.from_numpy(csr.data).to(device=device, dtype=dtype)
        self.col_ptr = torch.from_numpy(csc.indptr.astype(np.int32)).to(device)
        self.row_idx = torch.from_numpy(csc.indices.astype(np.int32)).to(device)
        self.vals_csc = torch.from_numpy(csc.data).to(device=device, dtype=dtype)
        blk_ptr, blk_pix, blk_vals = _actuator_blocks(csc, BLOCK_ACTUATORS)
        self.blk_ptr = torch.from_numpy(blk_ptr).to(device)
        self.blk_pix = torch.from_numpy(blk_pix).to(device)
        self.blk_vals = torch.from_numpy(blk_vals).to(device=device, dtype=dtype)

    def apply(self, coeffs):
        """surface[v, p] = sum_a M[p, a] coeffs[v, a] for coeffs of shape (..., nact)."""
        npix, nact = self.shape
        lead = tuple(coeffs.shape[:-1])
        c = _batched(coeffs.to(device=self.vals.device, dtype=self.dtype), nact)
        out = torch.empty(lead + (npix,), dtype=self.dtype, device=self.vals.device)
        if out.numel() == 0:
            return out
        rc = _lib.lib().hx_influence_apply(npix, nact, _lib.dptr(self.row_ptr), _lib.dptr(self.col_idx),
                                           _lib.dptr(self.vals), _lib.dtype_code(self.dtype), c.shape[0],
                                           _lib.dptr(c), _lib.dptr(out), _lib.stream_handle())
        _lib.check(rc, 'hx_influence_apply')
        return out

    def apply_transpose(self, g):
        """g_coeffs[v, a] = sum_p M[p, a] g[v, p] for g of shape (..., npix)."""
        npix, nact = self.shape
        lead = tuple(g.shape[:-1])
        g2 = _batched(g.to(device=self.vals.device, dtype=self.dtype), npix)
        out = torch.empty(lead + (nact,), dtype=self.dtype, device=self.vals.device)
        if out.numel() == 0:
            return out
        rc = _lib.lib().hx_influence_apply_transpose_blocked(npix, nact, _lib.dptr(self.blk_ptr),
                                                             _lib.dptr(self.blk_pix), _lib.dptr(self.blk_vals),
                                                             _lib.dtype_code(self.dtype), g2.shape[0], _lib.dptr(g2),
                                                             _lib.dptr(out), _lib.stream_handle())
        _lib.check(rc, 'hx_influence_apply_transpose_blocked')
        return out


BLOCK_ACTUATORS = 4  # actuators per block of the blocked transpose (kBA in csrc/influence.cu)


def _actuator_blocks(csc, block):
    """Union pixel lists of blocks of ``block`` consecutive actuators, from the CSC form: (block pointers
    (nblk + 1), pixel indices (sorted within a block), weights (n x block, zero where an actuator of the block does
    not reach the pixel))."""
    npix, nact = csc.shape
    nblk = -(-nact // block)
    ptr = np.zeros(nblk + 1, np.int32)
    pix, vals = [], []
    for b in range(nblk):
        a0, a1 = b * block, min(nact, (b + 1) * block)
        rows = csc.indices[csc.indptr[a0]:csc.indptr[a1]]
        u = np.unique(rows)
        w = np.zeros((u.size, block), csc.data.dtype)
        for a in range(a0, a1):
            r = csc.indices[csc.indptr[a]:csc.indptr[a + 1]]
            w[np.searchsorted(u, r), a - a0] = csc.data[csc.indptr[a]:csc.indptr[a + 1]]
        pix.append(u.astype(np.int32))
        vals.append(w)
        ptr[b + 1] = ptr[b] + u.size
    pix = np.concatenate(pix) if pix else np.zeros(0, np.int32)
    vals = np.concatenate(vals) if vals else np.zeros((0, block))
    return ptr, pix, np.ascontiguousarray(vals).reshape(-1)


def _weights(w, n, device):
    if w is None:
        return None
    w = w.data if hasattr(w, 'grid') and hasattr(w, 'data') else w
    w = torch.as_tensor(np.asarray(w) if not isinstance(w, torch.Tensor) else w)
    w = w.to(device=device, dtype=torch.float32).reshape(-1).contiguous()
    if w.numel() != n:
        raise ValueError('weights have %d points, the field %d' % (w.numel(), n))
    return w


def intensity_sums(e, w=None):
    """sum_p w[p] |e[..., p]|^2 per field in compensated float-float arithmetic, as a float64 tensor of e's batch
    shape (w: a real weight or region mask per point, or None)."""
    if e.dtype not in _REAL:
        raise TypeError('intensity sums take complex64 or complex128 fields, not %s' % e.dtype)
    n = e.shape[-1]
    lead = tuple(e.shape[:-1])
    batch = int(np.prod(lead)) if lead else 1
    out = torch.zeros(lead, dtype=torch.float64, device=e.device)
    if batch == 0 or n == 0:
        return out
    e2 = _batched(e, n)
    wt = _weights(w, n, e.device)
    lib = _lib.lib()
    nbytes = int(lib.hx_intensity_sums_workspace_bytes(n, batch))
    ws = _lib.workspace(nbytes, e.device)
    rc = lib.hx_intensity_sums(_lib.dptr(e2), _lib.dtype_code(e.dtype), n, batch,
                               None if wt is None else _lib.dptr(wt), _lib.dptr(out), _lib.dptr(ws), nbytes,
                               _lib.stream_handle())
    _lib.check(rc, 'hx_intensity_sums')
    return out


def intensity_sums_grad(e, w, g):
    """Gradient of ``intensity_sums`` in torch's convention: 2 g[b] w e_b, in e's dtype and shape."""
    n = e.shape[-1]
    lead = tuple(e.shape[:-1])
    batch = int(np.prod(lead)) if lead else 1
    out = torch.empty(lead + (n,), dtype=e.dtype, device=e.device)
    if batch == 0 or n == 0:
        return out
    e2 = _batched(e, n)
    wt = _weights(w, n, e.device)
    g2 = g.to(device=e.device, dtype=torch.float64).reshape(-1).contiguous()
    if g2.numel() != batch:
        raise ValueError('expected %d upstream gradients, got %d' % (batch, g2.numel()))
    rc = _lib.lib().hx_intensity_sums_grad(_lib.dptr(e2), _lib.dtype_code(e.dtype), n, batch,
                                           None if wt is None else _lib.dptr(wt), _lib.dptr(g2), _lib.dptr(out),
                                           _lib.stream_handle())
    _lib.check(rc, 'hx_intensity_sums_grad')
    return out
