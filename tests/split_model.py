"""numpy model of the split-operand tensor-core GEMM arithmetic (test helper).

It states what the tcgen05 kernel computes, step for step: the complex GEMM
as a real GEMM on [[Ar, -Ai], [Ai, Ar]] . [Br; Bi]; per-row (A) and per-column
(B) power-of-two scales; three fixed-point slices of widths (6, 11, 11) bits
rounded to nearest; the products of slice levels 0-3 (all but a2 b2); exact sums (float64 sums
of integer products are exact at these sizes, as the kernel's exact FP32 level-0
sums are).  The device result must agree with this model to float64 round-off
of the final combination, which pins the kernel bit for bit apart from the
FP32 rounding of the level-1/level-2 accumulators.
"""
import numpy as np

WIDTHS = (6, 11, 11)
LEVELS = 3


def _pow2_scale(mx):
    mx = np.where((mx > 0) & np.isfinite(mx), mx, 1.0)
    _, e = np.frexp(mx)
    return np.ldexp(1.0, e)


def _slices(X):
    """Row-wise slices of a real matrix X: X ~ scale * sum_p 2^-shift_p a_p."""
    scale = _pow2_scale(np.abs(X).max(axis=1, keepdims=True))
    t = X / scale
    out = []
    shift = 0
    for b in WIDTHS:
        shift += b
        t = t * 2.0**b
        a = np.rint(t)
        out.append((a, shift))
        t = t - a
    return scale, out


def split_matmul(A, B):
    """Complex A (m x k) @ B (k x n) as the split kernel computes it (float64 result)."""
    A = np.asarray(A, np.complex128)
    B = np.asarray(B, np.complex128)
    Ae = np.block([[A.real, -A.imag], [A.imag, A.real]])
    Be = np.vstack([B.real, B.imag])
    row_scale = _pow2_scale(np.maximum(np.abs(A.real), np.abs(A.imag)).max(axis=1, keepdims=True))
    col_scale = _pow2_scale(np.maximum(np.abs(B.real), np.abs(B.imag)).max(axis=0, keepdims=True))
    As = []
    t = Ae / np.vstack([row_scale, row_scale])
    shift = 0
    for b in WIDTHS:
        shift += b
        t = t * 2.0**b
        a = np.rint(t)
        As.append((a, shift))
        t = t - a
    Bs = []
    t = Be / col_scale
    shift = 0
    for b in WIDTHS:
        shift += b
        t = t * 2.0**b
        a = np.rint(t)
        Bs.append((a, shift))
        t = t - a
    C = np.zeros((Ae.shape[0], Be.shape[1]))
    for i, (a, sa) in enumerate(As):
        for j, (b, sb) in enumerate(Bs):
            if i + j <= LEVELS:
                C += (a @ b) * 2.0**(-sa - sb)
    C = C * np.vstack([row_scale, row_scale]) * col_scale
    m = A.shape[0]
    return C[:m] + 1j * C[m:]


def mft_forward(e, x, y, u, v, w_in):
    """Forward MFT with the split arithmetic: w_in * M1 . (E . M2)."""
    m1 = np.exp(-1j * np.outer(v, y))
    m2 = np.exp(-1j * np.outer(x, u))
    E = np.asarray(e, np.complex128).reshape(len(y), len(x))
    return (w_in * split_matmul(m1, split_matmul(E, m2))).ravel()
