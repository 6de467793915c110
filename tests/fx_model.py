"""Host restatement of the integer-unit restart combination
(ed_bv_mult_real with ED_RESTART_FIXED), used by the tests to check the
kernel bit for bit.  It follows the kernel's arithmetic exactly:

  * row r of V: E = the largest biased exponent of V[0..m-1][r];
    q = round-half-up(|v| 2^(1078 - E)) with the sign of v (|q| <= 2^56),
    0 for zeros and subnormals; a non-finite entry makes the row's outputs NaN;
  * column c of Y: F_c with max_i |Y[i][c]| < 2^F_c (0 for a zero column),
    y = round-half-away(Y 2^(56 - F_c));
  * T = sum_i q_i y_ic exactly, out = T 2^(E - 1078 + F_c - 56) rounded to
    nearest even (results below 2^-1022 flush to zero).
"""
import math
from fractions import Fraction

import numpy as np


def _fx56_row(v, E):
    b = int(np.float64(v).view(np.uint64))
    e = (b >> 52) & 0x7FF
    if e == 0:
        return 0
    mant = (b & ((1 << 52) - 1)) | (1 << 52)
    sh = e - E + 3
    if sh >= 0:
        q = mant << sh
    elif sh > -60:
        q = (mant + (1 << (-sh - 1))) >> (-sh)
    else:
        q = 0
    return -q if b >> 63 else q


def _round_away(x):
    f = Fraction(abs(x))
    i = int(f)
    if f - i >= Fraction(1, 2):
        i += 1
    return -i if x < 0 else i


def _to_double(T, X):
    if T == 0:
        return 0.0
    val = Fraction(T) * Fraction(2) ** X
    d = float(val)  # correctly rounded, ties to even
    return d if abs(d) >= 2.0 ** -1022 else 0.0


def restart_fixed(V, Y):
    """out (l, n) for V (m, n) and Y (m, l)."""
    V = np.asarray(V, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    m, n = V.shape
    l = Y.shape[1]
    yq = np.zeros((m, l), dtype=object)
    F = [0] * l
    for c in range(l):
        mx = float(np.abs(Y[:, c]).max())
        F[c] = math.frexp(mx)[1] if mx > 0 else 0
        for i in range(m):
            yq[i, c] = _round_away(Fraction(float(Y[i, c])) * Fraction(2) ** (56 - F[c]))
    out = np.empty((l, n))
    bits = V.view(np.uint64)
    for r in range(n):
        ex = [int((int(bits[i, r]) >> 52) & 0x7FF) for i in range(m)]
        E = max(ex)
        if E == 0x7FF:
            out[:, r] = np.nan
            continue
        q = [_fx56_row(V[i, r], E) for i in range(m)]
        for c in range(l):
            T = sum(q[i] * int(yq[i, c]) for i in range(m))
            out[c, r] = _to_double(T, E - 1078 + F[c] - 56)
    return out
