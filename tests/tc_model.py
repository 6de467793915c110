"""Host restatement of the exact-slice tensor-core restart combination
(ed_bv_mult_real with ED_RESTART_EXACT), used by the tests to check the
kernel bit for bit.  It follows the kernel's arithmetic exactly:

  * V in tiles of 128 rows; a tile's scale 2^P is the smallest power of two
    above its largest finite entry (P = largest biased exponent - 1022);
    q = round-half-up(|v| 2^(63 - P)), computed from the FP64 bits;
  * Y column c with scale 2^F_c (F_c from frexp of max_i |Y[i][c]|),
    yq = round-half-away(|y| 2^(63 - F_c));
  * eight signed 8-bit slices of each, level sums
    D_u = sum_i sum_{s+t=u} b_s d_t for u = 0..8 (exact integers);
  * T = sum_u D_u 2^(8(8-u)), out = T 2^(P + F_c - 78) rounded to nearest
    even (rows with a non-finite entry give NaN).
"""
import math
from fractions import Fraction

import numpy as np

ROWS = 128


def _slices(q, neg):
    """(..., 8) int64 signed slices, slice 0 the most significant byte."""
    sh = np.array([8 * (7 - s) for s in range(8)], dtype=np.uint64)
    b = ((q[..., None] >> sh) & np.uint64(0xFF)).astype(np.int64)
    return np.where(neg[..., None], -b, b)


def quantize_tiles(V):
    """V: (m, n) float64.  Returns (slices (m, n, 8) int64, P per row, bad rows)."""
    m, n = V.shape
    bits = np.ascontiguousarray(V).view(np.uint64)
    e = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    finite = e != 0x7FF
    bad = ~finite.all(axis=0)
    ef = np.where(finite, e, 0)
    ntile = (n + ROWS - 1) // ROWS
    pad = np.zeros((m, ntile * ROWS), dtype=np.int64)
    pad[:, :n] = ef
    E_tile = pad.reshape(m, ntile, ROWS).max(axis=(0, 2))
    E = np.repeat(E_tile, ROWS)[:n]
    mant = (bits & np.uint64((1 << 52) - 1)) | np.uint64(1 << 52)
    sh = e - E[None, :] + 10
    q = np.zeros((m, n), dtype=np.uint64)
    up = (sh >= 0) & (e != 0) & finite
    q[up] = mant[up] << sh[up].astype(np.uint64)
    dn = (sh < 0) & (sh > -64) & (e != 0) & finite
    rs = (-sh[dn]).astype(np.uint64)
    q[dn] = (mant[dn] + (np.uint64(1) << (rs - np.uint64(1)))) >> rs
    neg = (bits >> np.uint64(63)) != 0
    return _slices(q, neg), E - 1022, bad


def quantize_y(Y):
    """Y: (m, l).  Returns (slices (m, l, 8) int64, F per column)."""
    m, l = Y.shape
    F = np.zeros(l, dtype=np.int64)
    q = np.zeros((m, l), dtype=np.uint64)
    for c in range(l):
        mx = float(np.abs(Y[:, c]).max())
        F[c] = math.frexp(mx)[1] if mx > 0 else 0
        for i in range(m):
            v = Fraction(abs(float(Y[i, c]))) * Fraction(2) ** int(63 - F[c])
            iv = int(v)
            q[i, c] = np.uint64(iv + (1 if v - iv >= Fraction(1, 2) else 0))
    return _slices(q, np.signbit(Y)), F


def restart_exact(V, Y):
    """out (l, n): the kernel's result for V (m, n) and Y (m, l)."""
    Vs, P, bad = quantize_tiles(np.asarray(V, dtype=np.float64))
    Ys, F = quantize_y(np.asarray(Y, dtype=np.float64))
    m, n, _ = Vs.shape
    l = Ys.shape[1]
    T = np.zeros((n, l), dtype=object)
    for u in range(9):
        Du = np.zeros((n, l), dtype=np.int64)
        for s in range(8):
            t = u - s
            if 0 <= t <= 7:
                Du += np.einsum('ir,ic->rc', Vs[:, :, s], Ys[:, :, t])
        T = T + Du.astype(object) * (1 << (8 * (8 - u)))
    out = np.empty((l, n))
    for r in range(n):
        for c in range(l):
            x = int(T[r, c])
            out[c, r] = math.ldexp(float(x), int(P[r] + F[c] - 78)) if x else 0.0
    out[:, bad] = np.nan
    return out
