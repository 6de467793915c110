"""Batched disorder sweep (DisorderBatch / ed_batch_*) against the oracle and
against one-at-a-time solves.

Tolerances: per-realisation diagonal bit-exact (build_disorder semantics);
batched H.v within 1e-14 * ||x_b||_2 per column; eigenvalues within 1e-10
relative of the plain solver and of dense diagonalisation, residual <= tol.
"""
import numpy as np
import pytest

import oracle
from oracle import Model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def ed():
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300
    return lsquantumed_gb300


def _setup(ed, N, mag, B, J2=0.2, W=2.0, seed0=0):
    env = ed.Environment(nspins=N)
    b = ed.Basis(env, mag)
    lat = ed.chain1D(env)
    h = ed.Hamiltonian(env, b, lat, 1.0, 1.0, J2, J2)
    h.build_diag(env)
    h.build_off_diag(env)
    fields = np.stack([oracle.rd_hi(seed0 + k, N, -W, W) for k in range(B)])
    return env, b, h, fields


def test_batch_diag_and_apply(ed):
    import torch
    N, mag, B = 12, 1, 5
    env, b, h, fields = _setup(ed, N, mag, B)
    bt = ed.DisorderBatch(h, fields)
    D = bt.diagonal()
    X = np.stack([oracle.start_vector(10 + k, b.size) for k in range(B)], axis=1)
    Y = bt.apply(torch.from_numpy(np.ascontiguousarray(X))).cpu().numpy()
    for k in range(B):
        M = Model(0, N, 1, N, mag, 1.0, 1.0, 0.2, 0.2)
        M.build(3, fields[k])
        assert np.array_equal(D[:, k].view(np.uint64), M.diag().view(np.uint64)), k
        y_ref = M.apply(X[:, k])
        assert np.abs(Y[:, k] - y_ref).max() <= 1e-14 * np.linalg.norm(X[:, k]), k


def test_batch_solve_matches_plain_and_dense(ed):
    N, mag, B, nev = 12, 0, 6, 2
    env, b, h, fields = _setup(ed, N, mag, B)
    bt = ed.DisorderBatch(h, fields)
    res = bt.solve(nev=nev, ncv=16, tol=1e-10, seed=0)
    assert np.all(res['nconv'] >= nev)
    assert np.all(res['errs'] <= 1e-9)
    for k in range(B):
        M = Model(0, N, 1, N, mag, 1.0, 1.0, 0.2, 0.2)
        M.build(3, fields[k])
        ev = np.linalg.eigvalsh(M.dense())
        assert np.allclose(res['evals'][k], ev[:nev], rtol=1e-10, atol=0), (k, res['evals'][k], ev[:nev])
        # one-at-a-time solve with the same fields
        hk = ed.Hamiltonian(env, b, ed.chain1D(env), 1.0, 1.0, 0.2, 0.2)
        hk.build_diag(env)
        hk.build_off_diag(env)
        hk.build_disorder(env, fields[k])
        eps = ed.Solver.SolverInit(hk, nev, 16)
        ed.Solver.EPSSetTolerances(eps, 1e-10)
        ed.Solver.solve(env, eps)
        for i in range(nev):
            e, _ = ed.Solver.eigenvalue(eps, i)
            assert abs(e - res['evals'][k][i]) <= 1e-10 * abs(e)
        # eigenvector of the batch: unit norm, residual small
        v = bt.eigenvector(k, 0).cpu().numpy()
        assert abs(np.linalg.norm(v) - 1.0) < 1e-10
        r = M.apply(v) - res['evals'][k][0] * v
        assert np.linalg.norm(r) <= 1e-8 * abs(res['evals'][k][0])


@pytest.mark.parametrize('restart', ['fp64', 'pair'])
def test_batch_restart_arithmetic(ed, restart):
    """Both restart arithmetics (FP64 with exact integers; float pairs, the
    default for large blocks) give the dense spectrum within 1e-10 relative
    and residuals within tol, on a block with realisations converging at
    different restarts."""
    N, mag, B, nev = 12, 1, 9, 2
    env, b, h, fields = _setup(ed, N, mag, B, seed0=40)
    bt = ed.DisorderBatch(h, fields)
    bt.set_restart_arithmetic(restart)
    res = bt.solve(nev=nev, ncv=12, tol=1e-10, seed=3)
    assert np.all(res['nconv'] >= nev) and np.all(res['errs'] <= 1e-10)
    for k in range(B):
        M = Model(0, N, 1, N, mag, 1.0, 1.0, 0.2, 0.2)
        M.build(3, fields[k])
        ev = np.linalg.eigvalsh(M.dense())
        assert np.allclose(res['evals'][k], ev[:nev], rtol=1e-10, atol=0), (k, res['evals'][k], ev[:nev])
    with pytest.raises(ed.InvalidArgument):
        bt.set_restart_arithmetic('fp32')


def test_batch_hv_tiles_bit_identical(ed):
    """Every tile of the batched H.v (rows per CTA tile x threads per CTA)
    runs the same exact integer sums: H.v results bit-identical for each
    forced tile.  The fused per-CTA reductions (x^T y, ||y||^2) are summed in
    a tile-dependent order, so the batched solve's eigenvalues agree to
    1e-12 relative (and bit for bit when a tile is repeated); the autotuner
    settles on one of the tiles."""
    import torch
    N, mag, B, nev = 14, 1, 40, 2
    env, b, h, fields = _setup(ed, N, mag, B, seed0=60)
    rng = np.random.default_rng(9)
    X = torch.from_numpy(rng.standard_normal((b.size, B)) + 1j * rng.standard_normal((b.size, B))).cuda()
    ref, yref = None, None
    for rows, threads in ((4, 128), (8, 256), (16, 128), (32, 256), (4, 128), (0, 0)):
        bt = ed.DisorderBatch(h, fields)
        bt.set_hv_tile(rows, threads)
        if rows:
            Y = bt.apply(X).cpu().numpy()
            if yref is None:
                yref = Y
            assert np.array_equal(Y.view(np.uint64), yref.view(np.uint64)), (rows, threads)
        res = bt.solve(nev=nev, ncv=12, tol=1e-10, seed=3)
        assert np.all(res['nconv'] >= nev) and np.all(res['errs'] <= 1e-10)
        if ref is None:
            ref = res['evals']
            first = res['evals']
        assert np.allclose(res['evals'], ref, rtol=1e-12, atol=0), (rows, threads)
        if (rows, threads) == (4, 128):
            assert np.array_equal(res['evals'].view(np.uint64), first.view(np.uint64))
        got = bt.hv_tile()
        if rows:
            assert got == (rows, threads)
        else:
            assert got[0] in (4, 8, 16, 32) and got[1] in (128, 256), got
    with pytest.raises(ed.InvalidArgument):
        bt.set_hv_tile(5, 128)


def test_solve_batches_concurrent(ed):
    """Three sectors solved at once (ed_batch_solve_many, one environment and
    stream each) give bit-identical results to solving them one after
    another with the same H.v tile; two batches of one environment are
    refused."""
    N, B, nev = 12, 12, 2
    fields = np.stack([oracle.rd_hi(80 + k, N, -2.0, 2.0) for k in range(B)])
    bts, seq = [], []
    for mag in (0, 1, 2):
        env = ed.Environment(nspins=N)
        b = ed.Basis(env, mag)
        h = ed.Hamiltonian(env, b, ed.chain1D(env), 1.0, 1.0, 0.2, 0.2)
        h.build_diag(env)
        h.build_off_diag(env)
        one = ed.DisorderBatch(h, fields)
        one.set_hv_tile(8, 256)  # one tile: the fused reductions then sum in the same order
        seq.append(one.solve(nev=nev, ncv=12, tol=1e-10, seed=2))
        bts.append(ed.DisorderBatch(h, fields))
        bts[-1].set_hv_tile(8, 256)
    res = ed.solve_batches(bts, nev=nev, ncv=12, tol=1e-10, seed=2)
    for r, q in zip(res, seq):
        assert np.all(r['nconv'] >= nev) and np.all(r['errs'] <= 1e-10)
        assert np.array_equal(r['evals'].view(np.uint64), q['evals'].view(np.uint64))
        assert r['its'] == q['its'] and r['nhv'] == q['nhv']
    with pytest.raises(ed.InvalidArgument):
        ed.solve_batches([bts[0], ed.DisorderBatch(bts[0].hamilt, fields)], nev=nev)


def test_batch_cuda_graphs(ed):
    """Expansion sweeps replayed from CUDA graphs (ed_batch_set_graphs, the
    default) give the results of direct launches bit for bit with the same
    H.v tile, and the sweeps after the first run from graphs."""
    N, mag, B, nev = 14, 1, 40, 2
    env, b, h, fields = _setup(ed, N, mag, B, seed0=90)
    res = {}
    for g in (False, True):
        bt = ed.DisorderBatch(h, fields)
        bt.set_hv_tile(8, 256)
        bt.set_graphs(g)
        r = bt.solve(nev=nev, ncv=12, tol=1e-10, seed=3)
        assert np.all(r['nconv'] >= nev) and np.all(r['errs'] <= 1e-10)
        res[g] = (r, bt.graph_sweeps())
    assert res[False][1] == 0 and res[True][1] >= 1, (res[False][1], res[True][1])
    assert res[True][1] == res[True][0]['its'] - 1
    assert np.array_equal(res[True][0]['evals'].view(np.uint64), res[False][0]['evals'].view(np.uint64))
    assert res[True][0]['its'] == res[False][0]['its'] and res[True][0]['nhv'] == res[False][0]['nhv']


def test_batch_rejects_bad_input(ed):
    env, b, h, fields = _setup(ed, 8, 0, 2)
    with pytest.raises(ValueError):
        ed.DisorderBatch(h, fields[:, :5])
