"""CPU checks of tests/tc_model.py, the host restatement the tensor-core
restart kernel is compared with bit for bit: where the fixed-point forms are
exact and no slice level is dropped, the model must give the correctly
rounded value of sum_i V[i][r] Y[i][c] (exact rational arithmetic); in
general it stays within 2^-60 of the tile and column scales."""
from fractions import Fraction

import numpy as np

import fx_model
import tc_model


def test_model_exact_when_nothing_is_dropped():
    rng = np.random.default_rng(0)
    m, n, l = 16, 300, 8
    # entries with at most 20 significant bits below 2^-1: the fixed point is
    # exact, and slice products beyond level 8 are zero
    V = rng.integers(-2 ** 19, 2 ** 19, (m, n)) * 2.0 ** -20
    Y = rng.integers(-2 ** 19, 2 ** 19, (m, l)) * 2.0 ** -20
    V[:, 0] = 0.5 - 2.0 ** -20  # every tile's largest entry below 1/2
    out = tc_model.restart_exact(V, Y)
    for r in range(0, n, 37):
        for c in range(l):
            exact = sum(Fraction(float(V[i, r])) * Fraction(float(Y[i, c])) for i in range(m))
            assert out[c, r] == float(exact), (r, c)


def test_model_error_bound():
    rng = np.random.default_rng(1)
    m, n, l = 32, 400, 8
    V = np.linalg.qr(rng.standard_normal((n, m)))[0].T
    Y = np.linalg.qr(rng.standard_normal((m, m)))[0][:, :l]
    out = tc_model.restart_exact(V, Y)
    for r in range(0, n, 41):
        tile = slice((r // 128) * 128, min(n, (r // 128 + 1) * 128))
        sv = np.abs(V[:, tile]).max()
        for c in range(l):
            exact = sum(Fraction(float(V[i, r])) * Fraction(float(Y[i, c])) for i in range(m))
            err = abs(Fraction(out[c, r]) - exact)
            assert err <= Fraction(2.0 ** -60) * Fraction(sv) * Fraction(np.abs(Y[:, c]).max()) * 2 + \
                Fraction(2.0 ** -53) * abs(exact), (r, c, float(err))


def test_model_nonfinite_rows():
    V = np.ones((4, 200)) * 0.25
    V[2, 150] = np.nan
    out = tc_model.restart_exact(V, np.eye(4)[:, :2])
    assert np.isnan(out[:, 150]).all() and np.isfinite(np.delete(out, 150, axis=1)).all()
    assert (np.delete(out, 150, axis=1) == 0.25).all()


def test_fixed_model_error_bound():
    """The integer-unit restart (fx_model): exact products of 56-bit inputs,
    one rounding; within 2^-51 of max|V row| * max|Y column| plus the final
    rounding of the exact value."""
    rng = np.random.default_rng(2)
    m, n, l = 16, 120, 8
    V = np.linalg.qr(rng.standard_normal((n, m)))[0].T * np.exp2(rng.integers(-20, 5, n))[None, :]
    Y = np.linalg.qr(rng.standard_normal((m, m)))[0][:, :l]
    V[3, 7] = 0.0
    out = fx_model.restart_fixed(V, Y)
    for r in range(0, n, 7):
        sv = np.abs(V[:, r]).max()
        for c in range(l):
            exact = sum(Fraction(float(V[i, r])) * Fraction(float(Y[i, c])) for i in range(m))
            err = abs(Fraction(out[c, r]) - exact)
            bound = Fraction(2.0 ** -51) * Fraction(sv) * Fraction(np.abs(Y[:, c]).max()) + \
                Fraction(2.0 ** -53) * abs(exact)
            assert err <= bound, (r, c, float(err), float(bound))


def test_fixed_model_exact_inputs():
    """Inputs with few significant bits are represented exactly: the output
    is the correctly rounded exact value; a non-finite entry gives NaN."""
    rng = np.random.default_rng(4)
    m, n, l = 12, 40, 5
    V = rng.integers(-2 ** 20, 2 ** 20, (m, n)) * 2.0 ** -21
    Y = rng.integers(-2 ** 20, 2 ** 20, (m, l)) * 2.0 ** -22
    V[:, 5] = 0.0
    V[2, 9] = np.inf
    out = fx_model.restart_fixed(V, Y)
    for r in range(n):
        for c in range(l):
            if r == 9:
                assert np.isnan(out[c, r])
                continue
            exact = sum(Fraction(float(V[i, r])) * Fraction(float(Y[i, c])) for i in range(m))
            assert out[c, r] == float(exact), (r, c)
