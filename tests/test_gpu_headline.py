"""Parity at the sizes the benchmark configurations are quoted on.

  * 6x5 square lattice, N=30, J2=0.55, Sz=0 (155,117,520 states): sampled
    rows of the matrix-free H.v, for every launch variant the eigensolve can
    pick (run-time compiled kernels with three register budgets, plain and
    fused with x^T y, real and complex storage) and the static kernel,
    against the oracle's row-by-row restatement of get_elem_diag /
    get_coup_elems (include/hamiltonian.tmpl_func.hpp:350-426) with ranks
    from search_index (src/hamiltonian.cpp:9-27).  Basis and ranks at the
    sampled indices bit-exact.
  * 4x5 square lattice, N=20, J2=0.5, nev=10: eigenvalues against the
    oracle's Krylov-Schur on the explicit matrix, and all N^2 <S_i.S_j> of the
    ground state against the oracle's correlation restatement.
  * 4x3 copy of that lattice: DSF weights |<n|S^z_q|0>|^2 summed over each
    degenerate level, against an independent dense computation.
  * Chain N=20, J2=0.2, fields h_i ~ U[-2, 2] from seeds 0..7, Sz = 0, 1, 2
    through the batched sweep, against oracle solves one realisation at a
    time; and a 70-realisation batch at N=12 spanning three restart tiles.

Tolerances (each stated where it is asserted): H.v rows 1e-12 absolute with
|x_i| < 1 (the absolute row sum of this operator is at most 70, so 121 FP64
additions in the oracle are bounded by 121 * 2^-53 * 70 = 9.4e-13); basis and
ranks bit-exact; eigenvalues 1e-10 relative with residual <= tol;
correlations 1e-8; DSF weights 1e-10.
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


def _square(ed, N, lx, ly, mag, J1, D1, J2, D2):
    env = ed.Environment(nspins=N)
    b = ed.Basis(env, mag)
    lat = ed.square2D(env, lx, ly)
    h = ed.Hamiltonian(env, b, lat, J1, D1, J2, D2)
    h.build_diag(env)
    h.build_off_diag(env)
    return env, b, lat, h


def _c5_rows(b, N, lx, ly):
    """2^16 random rows, the first and last ranks, the checkerboard and
    column-stripe states, and the rows (from 2^18 more random ones) whose
    states have the most antiparallel bonds inside the low half, inside the
    high half and across the halves of the two-table rank split."""
    dim = b.size
    rng = np.random.default_rng(2030)
    rows = set(int(r) for r in rng.integers(0, dim, 1 << 16))
    rows |= {0, 1, 2, dim - 3, dim - 2, dim - 1}
    for f in (lambda x, y: (x + y) % 2 == 0, lambda x, y: (x + y) % 2 == 1,
              lambda x, y: x % 2 == 0, lambda x, y: x % 2 == 1):
        s = sum(1 << (x * ly + y) for x in range(lx) for y in range(ly) if f(x, y))
        if bin(s).count('1') == N // 2:
            rows.add(int(oracle.search_index(s, N)))
    nn, nnn = oracle.bond_pairs(1, N, lx, ly)
    pairs = np.concatenate([nn, nnn]).astype(np.uint64)
    half = min(14, (N + 1) // 2)
    lo = (pairs[:, 0] < half) & (pairs[:, 1] < half)
    hi = (pairs[:, 0] >= half) & (pairs[:, 1] >= half)
    ac = ~(lo | hi)
    cand = np.unique(rng.integers(0, dim, 1 << 18))
    st = b.search_elem(cand).astype(np.uint64)
    counts = {k: np.zeros(len(cand), np.int64) for k in ('lo', 'hi', 'ac')}
    for k0 in range(0, len(pairs), 8):
        p = pairs[k0:k0 + 8]
        anti = (((st[:, None] >> p[None, :, 0]) ^ (st[:, None] >> p[None, :, 1])) & np.uint64(1)).astype(np.int64)
        for name, m in (('lo', lo), ('hi', hi), ('ac', ac)):
            counts[name] += anti[:, m[k0:k0 + 8]].sum(axis=1)
    for name in counts:
        for r in cand[np.argsort(-counts[name], kind='stable')[:16]]:
            rows.add(int(r))
    return np.array(sorted(rows), dtype=np.int64)


def test_c5_hv_sampled_rows(ed):
    """N=30 6x5 J1-J2 (J2=0.55) Sz=0: 65,5xx sampled rows of H x against the
    oracle, 1e-12 absolute, for each H.v launch variant in real storage
    (plain and fused with x^T y / ||y||^2, whose sums must match torch's at
    1e-12 relative and whose y must equal the plain product bit for bit) and
    for the complex-storage kernel on a complex input."""
    import torch
    N, lx, ly = 30, 6, 5
    J1, D1, J2, D2 = 1.0, 1.0, 0.55, 0.55
    env, b, lat, h = _square(ed, N, lx, ly, 0, J1, D1, J2, D2)
    dim = b.size
    assert dim == 155117520
    rows = _c5_rows(b, N, lx, ly)
    # basis and ranks at the sampled indices, bit-exact
    st = b.search_elem(rows)
    ref_st = np.array([oracle.search_elem(int(r), N, N // 2) for r in rows], dtype=np.uint64)
    assert np.array_equal(st.astype(np.uint64), ref_st)
    assert np.array_equal(b.search_index(ref_st), rows)

    seed = 17
    tol = 1e-12
    x = torch.from_numpy(oracle.start_vector_r(seed, dim)).cuda()
    ref = oracle.rows_apply_seeded(1, N, lx, ly, 0, J1, D1, J2, D2, seed, rows)
    rows_t = torch.from_numpy(rows).cuda()
    y = torch.empty_like(x)
    yd = torch.empty_like(x)
    for v in ('auto', 'jit-b3', 'jit-b4', 'jit', 'jit-w3', 'jit-w4', 'u4-b6'):
        h.set_hv_variant(v)
        h.apply_real(x, out=y)
        err = np.abs(y[rows_t].cpu().numpy() - ref).max()
        assert err <= tol, (v, err)
        _, xy, yy = h.apply_real_dot(x, out=yd)
        assert torch.equal(yd.view(torch.int64), y.view(torch.int64)), v
        assert abs(xy - torch.dot(x, y).item()) <= 1e-12 * abs(xy), (v, xy)
        assert abs(yy - torch.dot(y, y).item()) <= 1e-12 * yy, (v, yy)
        if v == 'auto':
            chosen = (h.hv_variant(False), h.hv_variant(True))
    assert all(c.startswith('jit') or c.startswith('u') for c in chosen), chosen
    h.set_hv_variant('auto')
    del y, yd
    # complex storage, complex input (re and im parts of the seeded vector)
    xi = torch.from_numpy(oracle.start_vector(seed, dim).imag.copy()).cuda()
    xc = torch.complex(x, xi)
    del xi
    refc = oracle.rows_apply_seeded(1, N, lx, ly, 0, J1, D1, J2, D2, seed, rows, complex_x=True)
    yc = torch.empty_like(xc)
    for v in ('auto', 'jit-b4'):
        h.set_hv_variant(v)
        h.apply(xc, out=yc)
        err = np.abs(yc[rows_t].cpu().numpy() - refc).max()
        assert err <= tol, (v, err)
    h.set_hv_variant('auto')


def test_c2_eigenvalues_and_correlations_vs_oracle(ed):
    """4x5 J1-J2 (J2=0.5), nev=10, eps_tol=1e-9: every returned eigenvalue
    within 1e-10 relative of the oracle's Krylov-Schur spectrum (tol 1e-12,
    16 values), each counted at most as often as it occurs there, with every
    distinct level below the largest present; residuals <= 1e-9.  All 400
    <S_i.S_j> of the (non-degenerate) ground state within 1e-8 of the
    oracle's correlation restatement on its own ground state."""
    N, lx, ly = 20, 4, 5
    env, b, lat, h = _square(ed, N, lx, ly, 0, 1.0, 1.0, 0.5, 0.5)
    eps = ed.Solver.SolverInit(h, 10)
    ed.Solver.EPSSetTolerances(eps, 1e-9)
    nconv = ed.Solver.solve(env, eps)
    assert nconv >= 10
    ev, errs = zip(*[ed.Solver.eigenvalue(eps, i) for i in range(10)])
    ev, errs = np.array(ev), np.array(errs)
    assert np.all(errs <= 1e-9), errs
    M = Model(1, N, lx, ly, 0, 1.0, 1.0, 0.5, 0.5)
    M.build(3)
    r = M.eps_solve(nev=16, ncv=40, tol=1e-12, vectors=True)
    assert r['nconv'] >= 16
    ref = np.sort(r['evals'][:16])
    tolv = 1e-10 * np.abs(ref).max()
    used = np.zeros(len(ref), bool)
    for e in np.sort(ev):
        k = np.where(~used & (np.abs(ref - e) <= tolv))[0]
        assert len(k), (e, ref)
        used[k[0]] = True
    below = ref[ref <= ev.max() + tolv]
    levels = [below[0]] + [x2 for x1, x2 in zip(below[:-1], below[1:]) if x2 - x1 > 1e-8]
    for lv in levels:
        assert np.any(np.abs(ev - lv) <= tolv), ('missing level', lv)
    assert ref[1] - ref[0] > 0.1  # non-degenerate ground state
    _, psi, _ = ed.Solver.solution(eps, 0)
    C = ed.SiSj(env, b).AllPairs(psi)
    ed.Solver.SolverClean(eps)
    psi_ref = r['evecs'][int(np.argmin(r['evals']))]
    psi_ref = psi_ref / np.linalg.norm(psi_ref)
    for i in range(N):
        for j in range(N):
            want = M.expect(oracle.SISJ, i, j, psi_ref)
            assert abs(C[i, j] - want) <= 1e-8, (i, j, C[i, j], want)


def _multiplets(E, tol=1e-8):
    order = np.argsort(E)
    groups, cur = [], [order[0]]
    for a, c in zip(order[:-1], order[1:]):
        if E[c] - E[a] > tol:
            groups.append(cur)
            cur = []
        cur.append(c)
    groups.append(cur)
    return groups


def test_c2_dsf_weights_vs_oracle(ed):
    """4x3 copy of the 4x5 workload: DSF weights sum_{n in level}
    |sum_i e^{iq.r_i} c_{i,n}|^2 / N at the two wave vectors the benchmark
    reports (q = (pi, 2 pi k / ly) nearest pi, and (pi, 0)), summed over each
    degenerate level (gauge-invariant), against ||P_E S^z_q |0>||^2 formed
    from the oracle's S^z_i |0> and a dense diagonalisation.  With the dense
    eigenvectors as targets every level is checked (1e-10); through the
    device eigensolve (DynStructFactor, nev=10, tol 1e-12) the levels whose
    every copy was found are checked at 1e-10 and the others bounded above
    (a single-vector Krylov run can miss copies of a degenerate level)."""
    import torch
    N, lx, ly = 12, 4, 3
    env, b, lat, h = _square(ed, N, lx, ly, 0, 1.0, 1.0, 0.5, 0.5)
    M = Model(1, N, lx, ly, 0, 1.0, 1.0, 0.5, 0.5)
    M.build(3)
    w, V = np.linalg.eigh(M.dense())
    psi0 = V[:, 0].astype(np.complex128)
    pos = np.array([(i // ly, i % ly) for i in range(N)], dtype=np.float64)
    qs = [(np.pi, 2 * np.pi * round(ly / 2 - 0.5) / ly), (np.pi, 0.0)]
    szi = np.stack([M.sqz(i, psi0) for i in range(N)])  # S^z_i |0>

    def oracle_weight(q, members):
        vq = (np.exp(1j * (pos @ np.asarray(q))) @ szi) / np.sqrt(N)  # S^z_q |0>
        P = V[:, members]
        return float(np.sum(np.abs(P.conj().T @ vq) ** 2))

    nlev = 40
    vecs = torch.from_numpy(np.ascontiguousarray(V[:, :nlev].T.astype(np.complex128)))
    c = ed.Phys.dsf_coefficients(env, b, b, 0, psi0, vecs)
    for q in qs:
        wts = ed.Phys.dsf_weights(c, pos, q)
        for g in _multiplets(w[:nlev]):
            if max(g) == nlev - 1:
                continue  # a level cut by the window
            assert abs(wts[g].sum() - oracle_weight(q, g)) <= 1e-10, (q, g)
    # full device pipeline
    eps = ed.Solver.SolverInit(h, 1)
    ed.Solver.EPSSetTolerances(eps, 1e-12)
    ed.Solver.solve(env, eps)
    gs, psi, _ = ed.Solver.solution(eps, 0)
    ed.Solver.SolverClean(eps)
    data = ed.DSF_data(b0=b, b1=b, lat=lat, h0=h, h1=h, nev=10, path='.')
    ed.Solver.options = {'eps_tol': 1e-12}
    try:
        dE, cg = ed.Phys.DynStructFactor(env, data, gs, psi, 0, 'Sqz', write=False)
    finally:
        ed.Solver.options = {}
    E = dE + gs
    full = 0
    for q in qs:
        wts = ed.Phys.dsf_weights(cg, pos, q)
        for g in _multiplets(E):
            members = np.where(np.abs(w - E[g[0]]) <= 1e-8)[0]
            assert len(members) >= len(g)
            want = oracle_weight(q, members)
            got = wts[g].sum()
            if len(members) == len(g):
                assert abs(got - want) <= 1e-10, (q, E[g[0]], got, want)
                full += 1
            else:
                assert got <= want + 1e-10, (q, E[g[0]], got, want)
    assert full >= 4


def test_c3_batch_at_n20_vs_oracle(ed):
    """Chain N=20, J1=1, J2=0.2, h_i ~ U[-2, 2] (hi_init of seeds 0..7),
    sectors Sz = 0, 1, 2 (dims 184756, 167960, 125970): the batched sweep's
    two lowest levels (nev=2, tol 1e-9) within 1e-10 relative of the oracle's
    Krylov-Schur on each realisation's explicit matrix (tol 1e-12), residuals
    <= 1e-9."""
    N, seeds = 20, range(8)
    fields = np.stack([oracle.rd_hi(s, N, -2.0, 2.0) for s in seeds])
    env = ed.Environment(nspins=N)
    for mag in (0, 1, 2):
        b = ed.Basis(env, mag)
        h = ed.Hamiltonian(env, b, ed.chain1D(env), 1.0, 1.0, 0.2, 0.2)
        h.build_diag(env)
        h.build_off_diag(env)
        bt = ed.DisorderBatch(h, fields)
        res = bt.solve(nev=2, ncv=0, tol=1e-9, seed=0)
        assert np.all(res['nconv'] >= 2) and np.all(res['errs'] <= 1e-9), (mag, res['errs'])
        for k, s in enumerate(seeds):
            M = Model(0, N, 1, N, mag, 1.0, 1.0, 0.2, 0.2)
            M.build(3, fields[k])
            r = M.eps_solve(nev=2, tol=1e-12, vectors=False)
            ref = np.sort(r['evals'])[:2]
            assert np.allclose(res['evals'][k], ref, rtol=1e-10, atol=0), (mag, s, res['evals'][k], ref)
        del bt


@pytest.mark.parametrize('restart', ['fp64', 'pair'])
def test_batch_spans_restart_tiles(ed, restart):
    """70 realisations of the N=12 chain (Sz=1): the restart combination runs
    in tiles of 32 realisations, so this block has two full tiles and a
    partial third.  Both restart arithmetics give every realisation's dense
    spectrum within 1e-10 relative, residuals <= 1e-10."""
    N, mag, B = 12, 1, 70
    env = ed.Environment(nspins=N)
    b = ed.Basis(env, mag)
    h = ed.Hamiltonian(env, b, ed.chain1D(env), 1.0, 1.0, 0.2, 0.2)
    h.build_diag(env)
    h.build_off_diag(env)
    fields = np.stack([oracle.rd_hi(100 + k, N, -2.0, 2.0) for k in range(B)])
    bt = ed.DisorderBatch(h, fields)
    bt.set_restart_arithmetic(restart)
    res = bt.solve(nev=2, ncv=12, tol=1e-10, seed=5)
    assert np.all(res['nconv'] >= 2) and np.all(res['errs'] <= 1e-10)
    for k in range(B):
        M = Model(0, N, 1, N, mag, 1.0, 1.0, 0.2, 0.2)
        M.build(3, fields[k])
        ev = np.linalg.eigvalsh(M.dense())
        assert np.allclose(res['evals'][k], ev[:2], rtol=1e-10, atol=0), (k, res['evals'][k], ev[:2])
