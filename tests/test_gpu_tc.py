"""Exact-slice tensor-core contractions: the restart combination
(ed_bv_mult_real) and the Gram-Schmidt dot products (ed_bv_dot_real) with
ED_RESTART_EXACT (the solver's exact arithmetic mode).

The kernel is checked bit for bit against tests/tc_model.py, a host
restatement of its arithmetic in exact integers (quantisation per 128-row
tile, slice levels, one rounding); against FP64 (numpy) within 2^-52 of the
largest output norm-wise; and inside the eigensolve against the FP64 restart
(eigenvalues 1e-12 relative, residuals <= tol, orthonormal Ritz vectors) and
the reference's golden eigenvalues (1e-12).  The default FP64 restart is
checked beside them for every size of a partial last group of outputs.
"""
import numpy as np
import pytest

import oracle
import tc_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def ed():
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300
    return lsquantumed_gb300


@pytest.fixture(scope='module')
def env(ed):
    return ed.Environment(nspins=2)


def _orth(rng, n, m):
    return np.linalg.qr(rng.standard_normal((n, m)))[0]


def _run(ed, env, V, Y, arith='exact'):
    import torch
    Vt = [torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in V]
    out = ed.bv_mult_real(env, Vt, Y, arith=arith)
    return np.stack([o.cpu().numpy() for o in out])


def _check(ed, env, V, Y):
    got = _run(ed, env, V, Y)
    want = tc_model.restart_exact(V, Y)
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), (np.argwhere(~same)[:5], got[~same][:5], want[~same][:5])
    return got


def test_exact_restart_small_bit_exact(ed, env):
    """One partial tile (n = 100), m = 16, 8 outputs."""
    rng = np.random.default_rng(3)
    V = _orth(rng, 100, 16).T.copy()
    Y = _orth(rng, 16, 16)[:, :8].copy()
    got = _check(ed, env, V, Y)
    assert np.abs(got - Y.T @ V).max() <= 2.0 ** -52


@pytest.mark.parametrize('n,m,l', [(1000, 16, 8), (1000, 16, 5), (4099, 13, 8), (777, 32, 8), (300, 1, 1),
                                   (128 * 152 * 4 + 37, 16, 8), (2000, 24, 15)])
def test_exact_restart_bit_exact(ed, env, n, m, l):
    rng = np.random.default_rng(n + 7 * m + l)
    V = _orth(rng, n, m).T.copy()
    Y = _orth(rng, m, m)[:, :l].copy()
    got = _check(ed, env, V, Y)
    ref = Y.T @ V
    assert np.linalg.norm(got - ref) <= 2.0 ** -52 * max(1.0, np.linalg.norm(ref)), (n, m, l)


@pytest.mark.parametrize('m', [16, 5])
@pytest.mark.parametrize('l', [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 16, 17])
def test_fp64_restart_groups(ed, env, m, l):
    """The default restart combination (FP64 FMA beside exact integer
    products, arith='fp64') for every size of the last group of eight
    outputs: each output within an FMA chain's bound of the exact value,
    2^-49 sum_i |V_i Y_ic|, plus the 62-bit quantisation of the integer
    columns, m 2^-62 (orthonormal V and Y, so every entry is at most 1)."""
    rng = np.random.default_rng(100 * m + l)
    n = 3001
    V = _orth(rng, n, m).T.copy()
    Y = _orth(rng, m, m)[:, :min(l, m)]
    Y = np.hstack([Y] * ((l + m - 1) // m))[:, :l].copy()
    got = _run(ed, env, V, Y, arith='fp64')
    ref = (Y.T.astype(np.longdouble) @ V.astype(np.longdouble))
    scale = np.abs(Y.T) @ np.abs(V)
    err = np.abs(got.astype(np.longdouble) - ref).astype(np.float64)
    assert (err <= 2.0 ** -49 * scale + m * 2.0 ** -62).all(), (np.argwhere(err > 2.0 ** -49 * scale)[:5], err.max())


def test_exact_restart_dynamic_range_zeros_nan(ed, env):
    """Rows scaled over 2^-60 .. 2^20 (tile scales differ), exact zeros, and a
    non-finite entry, which makes its row's outputs NaN and nothing else."""
    rng = np.random.default_rng(5)
    n, m = 1500, 16
    V = rng.standard_normal((m, n)) * np.exp2(rng.integers(-60, 20, n))[None, :]
    V[:, 300:420] = 0.0
    V[3, 17] = 0.0
    V[5, 999] = np.inf
    Y = _orth(rng, m, m)[:, :8].copy()
    got = _check(ed, env, V, Y)
    assert np.isnan(got[:, 999]).all() and np.isfinite(np.delete(got, 999, axis=1)).all()
    assert (got[:, 300:420] == 0.0).all()


def test_exact_restart_arguments(ed, env):
    import torch
    V = [torch.zeros(64, dtype=torch.float64, device='cuda') for _ in range(33)]
    with pytest.raises(ed.EDError):
        ed.bv_mult_real(env, V, np.eye(33)[:, :4], arith='exact')  # m > 32
    with pytest.raises(ed.InvalidArgument):
        ed.bv_mult_real(env, V[:4], np.eye(4), out=[V[0], V[5], V[6], V[7]], arith='exact')  # aliasing
    with pytest.raises(ed.InvalidArgument):
        ed.bv_mult_real(env, V[:4], np.eye(4), arith='half')


def _solve(ed, env_, h, nev, tol, ncv, restart):
    eps = ed.Solver.SolverInit(h, nev, ncv)
    ed.Solver.EPSSetTolerances(eps, tol, 0)
    eps.set_restart_arithmetic(restart)
    nconv = ed.Solver.solve(env_, eps)
    st = eps.stats()
    ev = np.array([ed.Solver.eigenvalue(eps, i)[0] for i in range(st['nreported'])])
    er = np.array([ed.Solver.eigenvalue(eps, i)[1] for i in range(st['nreported'])])
    return eps, nconv, ev, er


def test_exact_restart_in_the_solve(ed):
    """4x6 J1-J2 (2.7M states), nev=4, ncv=16, tol 1e-10: the exact restart
    and the FP64 one give the same lowest levels to 1e-12 relative, residuals
    within tol, orthonormal Ritz vectors."""
    env_ = ed.Environment(nspins=24)
    b = ed.Basis(env_, 0)
    h = ed.Hamiltonian(env_, b, ed.square2D(env_, 4, 6), 1.0, 1.0, 0.55, 0.55)
    h.build_diag(env_)
    h.build_off_diag(env_)
    out = {}
    for mode in ('fp64', 'exact'):
        eps, nconv, ev, er = _solve(ed, env_, h, 4, 1e-10, 16, mode)
        assert nconv >= 4 and np.all(er[:4] <= 1e-10), (mode, er)
        X = np.stack([ed.Solver.solution(eps, i)[1].cpu().numpy().real for i in range(4)])
        ed.Solver.SolverClean(eps)
        assert np.abs(X @ X.T - np.eye(4)).max() <= 1e-12, mode
        out[mode] = ev[:4]
    assert np.allclose(out['exact'], out['fp64'], rtol=1e-12, atol=0), out


def test_exact_restart_golden_eigenvalues(ed, golden):
    """Every golden solver case of the reference with the exact restart
    forced: eigenvalues within 1e-12, residuals <= 1e-8."""
    from test_gpu_parity import _match_levels
    cache = {}
    for rec in golden['solver']:
        N = rec['N']
        if N not in cache:
            cache[N] = ed.Environment(nspins=N)
        env_ = cache[N]
        b = ed.Basis(env_, rec['mag'])
        lat = ed.chain1D(env_) if rec['ltype'] == 0 else ed.square2D(env_, rec['lx'], rec['ly'])
        h = ed.Hamiltonian(env_, b, lat, rec['J1'], rec['D1'], rec['J2'], rec['D2'])
        for c in rec['calls']:
            if c == 'build_diag':
                h.build_diag(env_)
            elif c == 'build_off_diag':
                h.build_off_diag(env_)
        want = max(i for i, _, _ in rec['expected']) + 1
        nev = max(want, rec['nev'])
        eps, nconv, ev, er = _solve(ed, env_, h, nev, 1e-12, min(max(2 * nev, nev + 15), b.size), 'exact')
        assert nconv >= want, rec['name']
        assert _match_levels(ev, rec['expected'], 1e-12), (rec['name'], ev, rec['expected'])
        assert np.all(er[:want] <= 1e-8), (rec['name'], er)
        ed.Solver.SolverClean(eps)


@pytest.mark.parametrize('n,m', [(100, 16), (5000, 16), (4099, 13), (3000, 20), (128 * 152 * 4 + 300, 16)])
def test_exact_dots(ed, env, n, m):
    """h = V^T w on the tensor cores (ed_bv_dot_real, exact slices) against
    the exact rational value: within 2^-52 |h| (the roundings at the end)
    plus the fixed-point quantisation, 2^-63 of each 128-row tile's largest
    entry per factor: 2^-62 sum_r (Mv_t |w_r| + Mw_t |v_r|) (FP64 FMA
    accumulates n roundings instead); the FP64 path beside it as a check of
    the harness."""
    import torch
    from fractions import Fraction
    rng = np.random.default_rng(n + m)
    V = _orth(rng, n, m).T.copy()
    w = rng.standard_normal(n) * np.exp2(rng.integers(-30, 3, n))
    w[50:70] = 0.0
    Vt = [torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in V]
    wt = torch.from_numpy(w).cuda()
    h = ed.bv_dot_real(env, Vt, wt, arith='exact')
    h64 = ed.bv_dot_real(env, Vt, wt, arith='fp64')
    idx = range(m) if n <= 5000 else (0, m - 1)
    def tile_max(x):
        t = np.zeros(((n + 127) // 128) * 128)
        t[:n] = np.abs(x)
        return np.repeat(t.reshape(-1, 128).max(axis=1), 128)[:n]
    Mw = tile_max(w)
    for i in idx:
        exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(V[i], w) if a and b)
        scale = float(np.abs(V[i] * w).sum())
        quant = float((tile_max(V[i]) * np.abs(w) + Mw * np.abs(V[i])).sum())
        err = abs(Fraction(float(h[i])) - exact)
        assert err <= Fraction(2.0 ** -52) * abs(exact) + Fraction(2.0 ** -62) * Fraction(quant), (i, float(err))
        assert abs(h64[i] - float(exact)) <= 1e-13 * scale, (i, h64[i], float(exact))
