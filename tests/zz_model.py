"""Host restatement of the S^z S^z sums of a real state (k_expect_zz_r with
k_expect_sym_finish, the path ed_expect_pairs takes for a real psi and
ED_OP_SZSZ / ED_OP_SISJ), used by the tests to check the kernel bit for bit.
It follows the kernel's arithmetic exactly:

  * w_r = psi_r * psi_r in FP64;
  * e with W = sum_r w_r < 2^e (W as the device sums it; the tests keep W
    away from powers of two, where the order of that sum could change e),
    S = 124 - e;
  * q_r = round-half-up(w_r 2^S) as an integer from the FP64 bits (0 for
    zeros and subnormals): exact for every w_r whose last bit is at or above
    2^-S;
  * T = sum_r q_r and, per pair (i, j), A = the sum of q_r over the rows
    whose spins i and j are antiparallel (exact integers), Z = T - 2 A;
  * out = 0.25 (d(Z) 2^-S), where d converts a 128-bit integer to FP64 as
    fma(double(hi), 2^64, double(lo)) on its magnitude; for S_i.S_i the
    kernel adds 0.5 (d(T) 2^-S).
"""
import math
from fractions import Fraction

import numpy as np


def basis_states(N, nup):
    """The fixed-Sz basis in rank order (ascending integers)."""
    from itertools import combinations
    out = [sum(1 << p for p in c) for c in combinations(range(N), nup)]
    return np.array(sorted(out), dtype=np.uint64)


def fx128(w, S):
    b = int(np.float64(w).view(np.uint64))
    E = (b >> 52) & 0x7FF
    if E == 0:
        return 0
    mant = (b & ((1 << 52) - 1)) | (1 << 52)
    sh = E - 1075 + S
    if sh >= 0:
        return mant << sh
    if sh > -54:
        return (mant + (1 << (-sh - 1))) >> (-sh)
    return 0


def _d(z):
    """The kernel's 128-bit integer to FP64 conversion."""
    neg = z < 0
    m = -z if neg else z
    hi, lo = m >> 64, m & ((1 << 64) - 1)
    v = float(Fraction(float(hi)) * 2 ** 64 + Fraction(float(lo)))  # one rounding, as fma
    return -v if neg else v


def scale_exponent(psi):
    W = math.fsum(float(x) * float(x) for x in psi)
    return math.frexp(W)[1] if W > 0 else 0


def szsz_sums(states, psi, pairs, e=None):
    """(Z per pair, T, S): the exact integer sums of the kernel."""
    if e is None:
        e = scale_exponent(psi)
    S = 124 - e
    q = [fx128(float(np.float64(x) * np.float64(x)), S) for x in psi]
    T = sum(q)
    st = [int(s) for s in states]
    Z = []
    for i, j in pairs:
        m = (1 << i) | (1 << j)
        A = 0
        for qr, s in zip(q, st):
            bits = s & m
            if bits != 0 and bits != m:
                A += qr
        Z.append(T - 2 * A)
    return Z, T, S


def szsz(states, psi, pairs, e=None):
    """<S^z_i S^z_j> for each pair as the kernel rounds it."""
    Z, T, S = szsz_sums(states, psi, pairs, e)
    inv = 2.0 ** -S
    return np.array([0.25 * (_d(z) * inv) for z in Z])
