"""CPU checks of tests/zz_model.py, the host restatement the real-state
S^z S^z kernel is compared with bit for bit: its sums are exact integers, so
each result must be within one final rounding (2^-52 relative) of the exact
rational value 0.25 sum_r w_r sigma_i sigma_j of the FP64 weights
w_r = fl(psi_r^2), also for a state whose weights span 60 binary orders."""
import math
from fractions import Fraction

import numpy as np

import zz_model


def _exact(states, psi, i, j):
    m = (1 << i) | (1 << j)
    t = Fraction(0)
    for s, x in zip(states, psi):
        w = Fraction(float(np.float64(x) * np.float64(x)))
        bits = int(s) & m
        t += -w if (bits != 0 and bits != m) else w
    return t / 4


def _check(states, psi, N):
    pairs = [(i, j) for i in range(N) for j in range(i, N)]
    got = zz_model.szsz(states, psi, pairs)
    for (i, j), g in zip(pairs, got):
        ex = _exact(states, psi, i, j)
        assert abs(Fraction(float(g)) - ex) <= Fraction(2.0 ** -52) * abs(ex), (i, j, g, float(ex))


def test_model_random_state():
    N, nup = 10, 5
    states = zz_model.basis_states(N, nup)
    rng = np.random.default_rng(3)
    psi = rng.standard_normal(len(states))
    psi *= math.sqrt(1.5) / np.linalg.norm(psi)  # sum of weights 1.5: far from a power of two
    _check(states, psi, N)


def test_model_wide_range_state():
    N, nup = 10, 4
    states = zz_model.basis_states(N, nup)
    rng = np.random.default_rng(4)
    psi = rng.standard_normal(len(states)) * np.exp2(-rng.integers(0, 30, len(states)))
    psi[0] = 1.2
    _check(states, psi, N)


def test_model_scale_and_bounds():
    """Every weight below 2^124 at the chosen scale, every sum too, and
    weights above 2^(e - 72) held exactly."""
    N, nup = 8, 4
    states = zz_model.basis_states(N, nup)
    psi = np.full(len(states), 2.0 ** -20)
    psi[0] = 1.0
    e = zz_model.scale_exponent(psi)
    Z, T, S = zz_model.szsz_sums(states, psi, [(0, 1), (2, 2)])
    assert S == 124 - e and 0 < T < 2 ** 124 and all(abs(z) <= T for z in Z)
    w = float(np.float64(2.0 ** -20) ** 2)
    assert zz_model.fx128(w, S) == Fraction(w) * 2 ** S
