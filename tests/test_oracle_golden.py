"""Pin the CPU oracle to the reference's own golden tests.

Every assertion here restates a known answer from the reference's
tests/unit_tests (extracted into tests/golden/reference_golden.json); the
entry's ``src`` field names the reference file it came from.
"""
import numpy as np
import pytest

from oracle import Model

NT = {0: 'nn', 1: 'nnn'}


def test_basis_layout_and_states(golden, orc):
    n = 0
    for rec in golden['basis']:
        size, ls, gs = orc.basis_layout(rec['N'], rec['mag'], rec['np'], rec['rank'])
        nup = rec['mag'] + rec['N'] // 2
        if 'size' in rec:
            assert size == rec['size'], rec
        if 'local_size' in rec:
            assert ls == rec['local_size'], rec
        if 'global_start_index' in rec:
            assert gs == rec['global_start_index'], rec
        if 'nspins_up' in rec:
            assert nup == rec['nspins_up'], rec
        if 'int_basis' in rec:
            got = orc.generate_basis(rec['N'], nup, gs, ls).tolist()
            assert got == rec['int_basis'], rec
            n += 1
    assert n >= 10


def test_basis_throw(golden, orc):
    for rec in golden['basis_throw']:
        with pytest.raises(ValueError):
            orc.basis_layout(rec['N'], rec['mag'], rec['np'], 0)


def test_int_basis_ref(golden, orc):
    r = golden['int_basis_ref']
    nup = r['mag'] + r['N'] // 2
    got = orc.generate_basis(r['N'], nup, 0, len(r['values'])).tolist()
    assert got == r['values']


def test_rank_unrank_roundtrip(orc):
    for N in (6, 8, 12, 16):
        for mag in range(-N // 2, N // 2 + 1):
            nup = mag + N // 2
            dim = orc.compute_size(N, nup)
            states = orc.generate_basis(N, nup, 0, dim)
            assert np.all(np.diff(states.astype(np.int64)) > 0)
            step = max(1, dim // 200)
            for r in range(0, dim, step):
                assert orc.search_index(int(states[r]), N) == r
                assert orc.search_elem(r, N, nup) == states[r]


def test_elem_diag(golden, orc):
    for rec in golden['elem_diag']:
        got = orc.get_elem_diag(rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['nt'], rec['state'])
        assert got == rec['expected'], rec


def test_disorder_elem(golden, orc):
    for rec in golden['disorder_elem']:
        N = rec['N']
        hi = np.arange(N, dtype=np.float64) / N
        got = orc.get_disorder_elem(rec['state'], N, hi)
        assert abs(got - rec['expected']) <= rec['tol'], rec


def test_coup_elems(golden, orc):
    checked = 0
    for rec in golden['coup_elems']:
        for r in rec['ranks']:
            got = orc.get_coup_elems(rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['np'], r,
                                     rec['nt'], rec['index'])
            if rec['ncol'] is not None:
                assert len(got) == rec['ncol'], rec
            assert got[:len(rec['cols'])] == rec['cols'], (rec, got)
            checked += 1
    assert checked >= 200


def _flags(calls):
    f = 0
    if 'build_diag' in calls:
        f |= Model.BUILD_DIAG
    if 'build_off_diag' in calls:
        f |= Model.BUILD_OFF_DIAG
    if 'build_disorder' in calls:
        f |= Model.BUILD_DISORDER
    return f


def _close_g(a, b):
    """PETSc ASCII viewers print %g (6 significant digits)."""
    return abs(a - b) <= 5e-6 * max(abs(a), abs(b)) + 1e-12


def test_matrices(golden, orc):
    for rec in golden['matrices']:
        M = Model(rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['J1'], rec['D1'], rec['J2'], rec['D2'])
        hi = np.arange(rec['N'], dtype=np.float64) / rec['N'] if rec['hi'] else None
        M.build(_flags(rec['calls']), hi)
        if rec['kind'] == 'diag_vec':
            d = M.diag()
            assert len(d) == len(rec['values']), rec['name']
            for a, b in zip(d, rec['values']):
                assert _close_g(a, b), (rec['name'], a, b)
        else:
            rp, cols, vals = M.csr()
            assert len(rec['rows']) == M.dim, rec['name']
            for r in range(M.dim):
                ref = rec['rows'][str(r)]
                got = [(int(c), float(v)) for c, v in zip(cols[rp[r]:rp[r + 1]], vals[rp[r]:rp[r + 1]])]
                assert [c for c, _ in got] == [c for c, _ in ref], (rec['name'], r, got, ref)
                for (c, v), (_, w) in zip(got, ref):
                    assert _close_g(v, w), (rec['name'], r, c, v, w)


@pytest.mark.parametrize('case', [
    (0, 12, 1, 12, 0, 1.0, 1.0, 0.0, 0.0),
    (1, 8, 2, 4, 1, 1.0, 0.3, 0.55, 0.2),   # 2x4: every bond appears twice
    (1, 12, 4, 3, 0, 1.0, 1.0, 0.5, 0.5),
    (1, 16, 4, 4, -2, 0.7, 1.3, 0.55, 0.55),
    (2, 12, 6, 2, 0, 1.0, 1.0, 0.5, 0.5),
    (1, 20, 4, 5, 0, 1.0, 1.0, 0.5, 0.5),
])
def test_rows_apply_matches_matrix(orc, case):
    """The row-by-row restatement (used at N=30, where no matrix fits) equals
    the explicit matrix built by the golden-pinned restatement on every row,
    to summation order (1e-13 absolute, |x_i| < 1), real and complex input."""
    ltype, N, lx, ly, mag, J1, D1, J2, D2 = case
    M = Model(ltype, N, lx, ly, mag, J1, D1, J2, D2)
    M.build(3)
    rows = np.arange(M.dim, dtype=np.int64)
    x = orc.start_vector(7, M.dim)
    got = orc.rows_apply_seeded(ltype, N, lx, ly, mag, J1, D1, J2, D2, 7, rows, complex_x=True)
    assert np.abs(got - M.apply(x)).max() <= 1e-13
    got_r = orc.rows_apply_seeded(ltype, N, lx, ly, mag, J1, D1, J2, D2, 7, rows)
    assert np.abs(got_r - M.apply(x.real.astype(np.complex128)).real).max() <= 1e-13
    assert np.array_equal(orc.start_vector_r(7, M.dim), x.real)


def _solve(M, nev, tol=1e-12):
    return M.eps_solve(nev=nev, ncv=max(2 * nev, nev + 15), tol=tol, seed=0)


def _match_levels(ev, expected, tol):
    """Expected values are the lowest eigenvalues either counted with
    multiplicity, or (when a single-vector Krylov run can only see one copy of
    a degenerate level, e.g. a diagonal matrix) as distinct levels."""
    idx = [i for i, _, _ in expected]
    vals = np.array([v for _, v, _ in expected])
    if np.all(np.abs(ev[idx] - vals) <= tol * np.maximum(1.0, np.abs(vals))):
        return True
    distinct = [ev[0]]
    for e in ev[1:]:
        if abs(e - distinct[-1]) > 1e-8:
            distinct.append(e)
    distinct = np.array(distinct)
    return len(distinct) > max(idx) and bool(
        np.all(np.abs(distinct[idx] - vals) <= tol * np.maximum(1.0, np.abs(vals))))


@pytest.mark.parametrize('idx', range(15))
def test_solver_eigenvalues(golden, orc, idx):
    if idx >= len(golden['solver']):
        pytest.skip('no case')
    rec = golden['solver'][idx]
    M = Model(rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['J1'], rec['D1'], rec['J2'], rec['D2'])
    M.build(_flags(rec['calls']))
    want = max(i for i, _, _ in rec['expected']) + 1
    if M.dim <= 3000:
        ev = np.linalg.eigvalsh(M.dense())
        assert _match_levels(ev, rec['expected'], 1e-12), (rec['name'], ev[:want + 2], rec['expected'])
    res = _solve(M, max(want, rec['nev']))
    assert res['nconv'] >= want
    assert _match_levels(res['evals'], rec['expected'], 1e-12), (rec['name'], res['evals'], rec['expected'])
    for i in range(want):
        assert res['errs'][i] <= 1e-8


def test_correlations(golden, orc):
    ops = {'SzSz': orc.SZSZ, 'SpSm': orc.SPSM}
    for rec in golden['correlation']:
        M = Model(rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['J1'], rec['D1'], rec['J2'], rec['D2'])
        M.build(3)
        res = _solve(M, 1)
        if rec['E0'] is not None:
            assert abs(res['evals'][0] - rec['E0']) <= 1e-12 * abs(rec['E0'])
        psi = res['evecs'][0]
        for i, j, v, tol in rec['pairs']:
            got = M.expect(ops[rec['op']], i, j, psi)
            assert abs(got.real - v) <= tol, (rec['name'], i, j, got, v)


def test_random_disorder(golden, orc):
    r = golden['random']
    seeds = orc.rd_seeds(r['reprod'], r['rep'])
    assert seeds.tolist() == r['seeds']
    hi = orc.rd_hi(int(seeds[r['hi_index']]), r['nspins'], r['min'], r['max'])
    assert np.allclose(hi, r['hi'], atol=r['tol'], rtol=0)


def _levels(evals, tol=1e-8):
    groups, cur = [], [0]
    for k in range(1, len(evals)):
        if abs(evals[k] - evals[cur[-1]]) < tol:
            cur.append(k)
        else:
            groups.append(cur)
            cur = [k]
    groups.append(cur)
    return groups


def test_dsf_reference_files(golden, orc):
    """dsf_d0_{1,2}.ref: energies E_n - E0 match; for non-degenerate levels the
    signed coefficients Re c_{n,i} are proportional (one phase factor per n)
    to c_{n,i} computed from real-phase eigenvectors."""
    for rec in golden['dsf']:
        M0 = Model(rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag0'], rec['J1'], rec['D1'], rec['J2'], rec['D2'])
        M0.build(3)
        gs = _solve(M0, 1)
        E0 = gs['evals'][0]
        assert abs(E0 - rec['GS']) <= 1e-12
        psi = gs['evecs'][0]
        M1 = M0 if rec['mag1'] == rec['mag0'] else Model(rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag1'],
                                                           rec['J1'], rec['D1'], rec['J2'], rec['D2'])
        if M1 is not M0:
            M1.build(3)
        H1 = M1.dense()
        ev, V = np.linalg.eigh(H1)
        nev = rec['nev']
        ref_E = np.array([row[0] for row in rec['spins'][0]])
        assert np.allclose(ev[:nev] - E0, ref_E, atol=1e-10), (ev[:nev] - E0, ref_E)
        # phase of the reference ground state is arbitrary; make ours real
        c = np.zeros((rec['N'], nev), dtype=np.complex128)
        for i in range(rec['N']):
            rhs = M0.sqz(i, psi) if rec['op'] == 'Sqz' else M0.sqp(M1, i, psi)
            for n in range(nev):
                c[i, n] = orc.vecdot(rhs, V[:, n])
        ph = np.exp(-1j * np.angle(c[np.unravel_index(np.argmax(abs(c)), c.shape)]))
        for grp in _levels(ev[:nev]):
            if len(grp) != 1:
                continue
            n = grp[0]
            ref = np.array([rec['spins'][i][n][1] for i in range(rec['N'])])
            ours = (c[:, n] * ph).real if np.abs((c[:, n] * ph).imag).max() < 1e-10 else np.abs(c[:, n])
            if np.abs(ref).max() < 1e-8:
                assert np.abs(ours).max() < 1e-8 or np.abs(ref).max() < 1e-8
                continue
            k = np.dot(ref, ours) / np.dot(ours, ours)
            assert abs(k) <= 1 + 1e-8
            assert np.allclose(ref, k * ours, atol=1e-9), (rec['name'], n, ref, ours)


def test_oracle_dsf_sum_rule():
    """The S(q, w) restatement satisfies the notebooks' sum rule
    (dynamicStep2_plotSw.ipynb cell 12: sum_{q,w} S dw / 2 pi = 1/4) on the
    oracle's full Sz=0 spectrum of an N=8 chain.  The window is widened to
    w in [-40, 40] so that the Lorentzian tails (half width 1/N) stay inside:
    the missing weight is then below 2e-3."""
    import oracle
    from oracle import Model
    N = 8
    M = Model(0, N, 1, N, 0, 1.0, 1.0, 0.0, 0.0)
    M.build(3)
    w, V = np.linalg.eigh(M.dense())
    psi0 = V[:, 0].astype(np.complex128)
    c = np.array([[np.vdot(V[:, n], M.sqz(i, psi0)) for n in range(len(w))] for i in range(N)])
    assert np.allclose(np.sum(np.abs(c) ** 2, axis=1), 0.25)  # <0|(S^z_i)^2|0> = 1/4
    S = oracle.dsf_average([oracle.dsf_spectrum(c, w - w[0], [(0, i) for i in range(N)],
                                                oracle.q_grid(N, 1, N), nw=160001, w_min=-40.0, w_max=40.0)])
    assert abs(oracle.dsf_sum_rule(S, -40.0, 40.0) - 0.25) < 2e-3
