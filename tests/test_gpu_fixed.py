"""Restart combination on the integer units (ed_bv_mult_real with
ED_RESTART_FIXED, the solver's 'fixed' restart arithmetic).

The kernel is checked bit for bit against tests/fx_model.py, a host
restatement of its arithmetic in exact integers (56-bit fixed point per row
of V and per column of Y, exact products, one rounding); against FP64
(numpy) norm-wise; and inside the eigensolve against the FP64 restart
(eigenvalues 1e-12 relative, residuals <= tol, orthonormal Ritz vectors) and
the reference's golden eigenvalues (1e-12).
"""
import numpy as np
import pytest

import fx_model

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


def _run(ed, env, V, Y, arith='fixed'):
    import torch
    Vt = [torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in V]
    out = ed.bv_mult_real(env, Vt, Y, arith=arith)
    return np.stack([o.cpu().numpy() for o in out])


def _check(ed, env, V, Y):
    got = _run(ed, env, V, Y)
    want = fx_model.restart_fixed(V, Y)
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), (np.argwhere(~same)[:5], got[~same][:5], want[~same][:5])
    return got


@pytest.mark.parametrize('n,m,l', [(100, 16, 8), (1000, 16, 5), (777, 13, 11), (300, 1, 1), (2000, 24, 15),
                                   (500, 32, 8), (128 * 152 * 4 + 37, 16, 8)])
def test_fixed_restart_bit_exact(ed, env, n, m, l):
    rng = np.random.default_rng(n + 7 * m + l)
    V = _orth(rng, n, m).T.copy()
    Y = _orth(rng, m, m)[:, :l].copy()
    if n > 20000:  # the model is pure Python: check a sample of the rows
        idx = np.r_[0:300, n - 300:n]
        got = _run(ed, env, V, Y)[:, idx]
        want = fx_model.restart_fixed(V[:, idx], Y)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
        got_all = _run(ed, env, V, Y)
    else:
        got_all = _check(ed, env, V, Y)
    ref = Y.T @ V
    assert np.linalg.norm(got_all - ref) <= 2.0 ** -50 * max(1.0, np.linalg.norm(ref)), (n, m, l)


def test_fixed_restart_dynamic_range_zeros_nan(ed, env):
    """Rows scaled over 2^-60 .. 2^20, exact zeros, a zero coefficient
    column, and a non-finite entry, which makes its row's outputs NaN and
    nothing else."""
    rng = np.random.default_rng(5)
    n, m = 1500, 16
    V = rng.standard_normal((m, n)) * np.exp2(rng.integers(-60, 20, n))[None, :]
    V[:, 300:420] = 0.0
    V[3, 17] = 0.0
    V[5, 999] = np.inf
    Y = _orth(rng, m, m)[:, :8].copy()
    Y[:, 6] = 0.0
    got = _check(ed, env, V, Y)
    assert np.isnan(got[:, 999]).all() and np.isfinite(np.delete(got, 999, axis=1)).all()
    assert (got[:, 300:420] == 0.0).all() and (np.delete(got[6], 999) == 0.0).all()


def _solve(ed, env_, h, nev, tol, ncv, restart):
    eps = ed.Solver.SolverInit(h, nev, ncv)
    ed.Solver.EPSSetTolerances(eps, tol, 0)
    eps.set_restart_arithmetic(restart)
    nconv = ed.Solver.solve(env_, eps)
    st = eps.stats()
    ev = np.array([ed.Solver.eigenvalue(eps, i)[0] for i in range(st['nreported'])])
    er = np.array([ed.Solver.eigenvalue(eps, i)[1] for i in range(st['nreported'])])
    return eps, nconv, ev, er


def test_fixed_restart_in_the_solve(ed):
    """4x6 J1-J2 (2.7M states), nev=4, ncv=16, tol 1e-10: the integer-unit
    restart and the FP64 one give the same lowest levels to 1e-12 relative,
    residuals within tol, orthonormal Ritz vectors."""
    env_ = ed.Environment(nspins=24)
    b = ed.Basis(env_, 0)
    h = ed.Hamiltonian(env_, b, ed.square2D(env_, 4, 6), 1.0, 1.0, 0.55, 0.55)
    h.build_diag(env_)
    h.build_off_diag(env_)
    out = {}
    for mode in ('fp64', 'fixed'):
        eps, nconv, ev, er = _solve(ed, env_, h, 4, 1e-10, 16, mode)
        assert nconv >= 4 and np.all(er[:4] <= 1e-10), (mode, er)
        X = np.stack([ed.Solver.solution(eps, i)[1].cpu().numpy().real for i in range(4)])
        ed.Solver.SolverClean(eps)
        assert np.abs(X @ X.T - np.eye(4)).max() <= 1e-12, mode
        out[mode] = ev[:4]
    assert np.allclose(out['fixed'], out['fp64'], rtol=1e-12, atol=0), out


def test_fixed_restart_golden_eigenvalues(ed, golden):
    """Every golden solver case of the reference with the integer-unit
    restart: eigenvalues within 1e-12, residuals <= 1e-8."""
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
        eps, nconv, ev, er = _solve(ed, env_, h, nev, 1e-12, min(max(2 * nev, nev + 15), b.size), 'fixed')
        assert nconv >= want, rec['name']
        assert _match_levels(ev, rec['expected'], 1e-12), (rec['name'], ev, rec['expected'])
        assert np.all(er[:want] <= 1e-8), (rec['name'], er)
        ed.Solver.SolverClean(eps)


def test_fixed_restart_arguments(ed, env):
    import torch
    V = [torch.zeros(64, dtype=torch.float64, device='cuda') for _ in range(4)]
    with pytest.raises(ed.InvalidArgument):
        ed.bv_mult_real(env, V, np.eye(4), out=[V[0], V[1], V[2], V[3]], arith='fixed')  # aliasing
    Y = np.eye(4)
    Y[1, 1] = np.nan
    with pytest.raises(ed.InvalidArgument):
        ed.bv_mult_real(env, V, Y, arith='fixed')
