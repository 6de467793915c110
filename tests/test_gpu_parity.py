"""Parity of the CUDA path (through the C ABI) with the CPU oracle and the
reference's golden vectors.

Tolerances (stated per test): basis, ranks and every matrix element are
bit-exact; H.v agrees to 1e-14 * ||x||_2 (max-norm of the difference);
eigenvalues to 1e-12 relative with residual <= 1e-8; correlations to the
golden tests' own 5e-10 / 5e-9.
"""
import numpy as np
import pytest

import oracle
from oracle import Model

pytestmark = pytest.mark.gpu

FLAGS = {'build_diag': 1, 'build_off_diag': 2, 'build_disorder': 4}


@pytest.fixture(scope='module')
def ed():
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300
    return lsquantumed_gb300


@pytest.fixture(scope='module')
def envs(ed):
    cache = {}

    def get(n):
        if n not in cache:
            cache[n] = ed.Environment(nspins=n)
        return cache[n]
    return get


def lattice(ed, env, ltype, lx, ly):
    if ltype == 0:
        return ed.chain1D(env)
    if ltype == 1:
        return ed.square2D(env, lx, ly)
    return ed.honeycomb2D(env, lx, ly)


def make_pair(ed, envs, ltype, N, lx, ly, mag, J1, D1, J2, D2, calls=('build_diag', 'build_off_diag'), hi=None):
    env = envs(N)
    b = ed.Basis(env, mag)
    lat = lattice(ed, env, ltype, lx, ly)
    h = ed.Hamiltonian(env, b, lat, J1, D1, J2, D2)
    flags = 0
    for c in calls:
        flags |= FLAGS[c]
        if c == 'build_diag':
            h.build_diag(env)
        elif c == 'build_off_diag':
            h.build_off_diag(env)
        elif c == 'build_disorder':
            h.build_disorder(env, hi)
    M = Model(ltype, N, lx, ly, mag, J1, D1, J2, D2)
    M.build(flags, hi)
    return env, b, h, M


# ---------------------------------------------------------------------------
# basis / ranks (bit-exact)
# ---------------------------------------------------------------------------
def test_basis_all_sectors_bit_exact(ed, envs):
    for N in range(2, 18, 2):
        env = envs(N)
        for mag in range(-N // 2, N // 2 + 1):
            b = ed.Basis(env, mag)
            nup = mag + N // 2
            assert b.size == oracle.compute_size(N, nup)
            ref = oracle.generate_basis(N, nup, 0, b.size)
            assert np.array_equal(b.int_basis, ref), (N, mag)
            assert np.array_equal(b.search_index(ref), np.arange(b.size)), (N, mag)
            idx = np.arange(0, b.size, max(1, b.size // 97))
            assert np.array_equal(b.search_elem(idx), ref[idx])


def test_basis_large_sectors(ed, envs):
    for N, mag in ((20, 0), (20, 1), (20, 2), (24, 0)):
        b = ed.Basis(envs(N), mag)
        ref = oracle.generate_basis(N, mag + N // 2, 0, b.size)
        assert np.array_equal(b.int_basis, ref)


def test_basis_golden_rank_slices(ed, envs, golden):
    for rec in golden['basis']:
        if 'int_basis' not in rec:
            continue
        size, ls, gs = oracle.basis_layout(rec['N'], rec['mag'], rec['np'], rec['rank'])
        b = ed.Basis(envs(rec['N']), rec['mag'])
        assert b.int_basis[gs:gs + ls].tolist() == rec['int_basis'], rec


def test_basis_invalid(ed, envs):
    env = envs(6)
    with pytest.raises(ValueError):
        ed.Basis(env, 4)
    with pytest.raises(ValueError):
        ed.Basis(env, -4)
    with pytest.raises(ValueError):
        ed.Environment(nspins=7)
    with pytest.raises(ed.EDError):
        ed.Basis(envs(34), 0)  # beyond the device path (N <= 32)
    b = ed.Basis(env, 0)
    with pytest.raises(ValueError):
        b.search_index(np.array([0b111111], dtype=np.uint64))  # wrong sector


# ---------------------------------------------------------------------------
# matrix elements (bit-exact against the oracle; %g against the golden dumps)
# ---------------------------------------------------------------------------
def _csr_equal(h, M):
    rp, cols, vals = h.export_csr()
    orp, ocols, ovals = M.csr()
    assert np.array_equal(rp, orp)
    assert np.array_equal(cols, ocols)
    assert np.array_equal(vals.view(np.uint64), ovals.view(np.uint64))  # bit-exact
    return rp, cols, vals


def test_golden_matrices(ed, envs, golden):
    for rec in golden['matrices']:
        hi = np.arange(rec['N'], dtype=np.float64) / rec['N'] if rec['hi'] else None
        env, b, h, M = make_pair(ed, envs, rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['J1'],
                                 rec['D1'], rec['J2'], rec['D2'], rec['calls'], hi)
        d = h.diagonal()
        assert np.array_equal(d.view(np.uint64), M.diag().view(np.uint64)), rec['name']
        if rec['kind'] == 'diag_vec':
            for a, v in zip(d, rec['values']):
                assert abs(a - v) <= 5e-6 * max(abs(a), abs(v)) + 1e-12, rec['name']
        else:
            rp, cols, vals = _csr_equal(h, M)
            for r in range(b.size):
                ref = rec['rows'][str(r)]
                got = list(zip(cols[rp[r]:rp[r + 1]].tolist(), vals[rp[r]:rp[r + 1]].tolist()))
                assert [c for c, _ in got] == [c for c, _ in ref], (rec['name'], r)
                for (_, v), (_, w) in zip(got, ref):
                    assert abs(v - w) <= 5e-6 * max(abs(v), abs(w)) + 1e-12, (rec['name'], r)


@pytest.mark.parametrize('case', [
    (0, 14, 1, 14, 0, 1.0, 1.0, 0.2, 0.2),
    (1, 16, 4, 4, 0, 1.0, 1.0, 0.5, 0.5),
    (1, 16, 4, 4, 1, 1.0, -0.43, -1.0, 1.0),
    (1, 12, 3, 4, 2, 0.7, 1.3, 0.35, 0.0),
    (1, 8, 2, 4, 0, 1.0, 1.0, 1.0, 1.0),  # duplicated bonds (lx = 2)
    (2, 12, 6, 2, 1, 1.0, 1.0, 0.5, 0.5),
    (1, 20, 4, 5, 0, 1.0, 1.0, 0.5, 0.5),
])
def test_csr_bit_exact(ed, envs, case):
    ltype, N, lx, ly, mag, J1, D1, J2, D2 = case
    env, b, h, M = make_pair(ed, envs, ltype, N, lx, ly, mag, J1, D1, J2, D2)
    _csr_equal(h, M)


def test_disorder_diagonal_bit_exact(ed, envs):
    for seed in (0, 3, 511):
        hi = oracle.rd_hi(seed, 20, -2.0, 2.0)
        env, b, h, M = make_pair(ed, envs, 0, 20, 1, 20, 1, 1.0, 1.0, 0.2, 0.2,
                                 ('build_diag', 'build_off_diag', 'build_disorder'), hi)
        assert np.array_equal(h.diagonal().view(np.uint64), M.diag().view(np.uint64))
        _csr_equal(h, M)


def test_per_bond_bit_exact(ed, envs):
    N = 16
    nn, nnn = oracle.bond_pairs(1, N, 4, 4)
    pairs = np.concatenate([nn, nnn])
    z = oracle.normal(5, len(pairs))
    J = np.where(np.arange(len(pairs)) < len(nn), 1.0, 0.5) * (1 + 0.1 * z)
    D = J.copy()
    hi = oracle.rd_hi(9, N, -0.5, 0.5)
    env = envs(N)
    b = ed.Basis(env, 0)
    h = ed.Hamiltonian.from_bonds(env, b, pairs, J, D)
    h.build_diag(env)
    h.build_off_diag(env)
    h.build_disorder(env, hi)
    M = Model(1, N, 4, 4, 0, bonds=pairs, Jb=J, Db=D)
    M.build(7, hi)
    _csr_equal(h, M)


# ---------------------------------------------------------------------------
# H.v (matrix-free and CSR) within 1e-14 * ||x||_2
# ---------------------------------------------------------------------------
@pytest.mark.parametrize('case', [
    (0, 6, 1, 6, 0, 1.0, 1.0, 0.0, 0.0),
    (0, 8, 1, 8, -2, 1.0, -1.4, 0.0, 0.0),
    (0, 12, 1, 12, 0, 1.0, 1.0, 0.0, 0.0),
    (1, 12, 3, 4, 0, 1.0, 1.0, 0.5, 0.5),
    (1, 16, 4, 4, 0, 1.0, 1.0, 0.5, 0.5),
    (1, 16, 4, 4, 3, 1.0, 0.3, 0.55, 0.55),
    (1, 20, 4, 5, 0, 1.0, 1.0, 0.5, 0.5),
    (0, 20, 1, 20, 2, 1.0, 1.0, 0.2, 0.2),
    (2, 12, 6, 2, 0, 1.0, 1.0, 0.5, 0.5),
])
def test_hv_matches_oracle(ed, envs, case):
    ltype, N, lx, ly, mag, J1, D1, J2, D2 = case
    env, b, h, M = make_pair(ed, envs, ltype, N, lx, ly, mag, J1, D1, J2, D2)
    for acc in ('exact', 'fixed64', 'fp64'):
        h.set_accumulation(acc)
        for seed in (1, 2):
            x = oracle.start_vector(seed, b.size)
            tol = 1e-14 * np.linalg.norm(x)
            y_ref = M.apply(x)
            y = h.apply(x).cpu().numpy()
            assert np.abs(y - y_ref).max() <= tol, (case, acc, np.abs(y - y_ref).max(), tol)
            assert np.abs(h.apply_host(x) - y_ref).max() <= tol
    # wide dynamic range and exact zeros in the input
    x = oracle.start_vector(3, b.size) * np.exp(np.linspace(-30, 5, b.size))
    x[::7] = 0.0
    y_ref = M.apply(x)
    for acc in ('exact', 'fixed64', 'fp64'):
        h.set_accumulation(acc)
        assert np.abs(h.apply(x).cpu().numpy() - y_ref).max() <= 1e-14 * np.linalg.norm(x), acc
    h.set_mode('csr')
    y2 = h.apply(x).cpu().numpy()
    assert np.abs(y2 - y_ref).max() <= tol


def test_hv_disorder_and_per_bond(ed, envs):
    hi = oracle.rd_hi(11, 20, -2.0, 2.0)
    env, b, h, M = make_pair(ed, envs, 0, 20, 1, 20, 0, 1.0, 1.0, 0.2, 0.2,
                             ('build_diag', 'build_off_diag', 'build_disorder'), hi)
    x = oracle.start_vector(3, b.size)
    assert np.abs(h.apply(x).cpu().numpy() - M.apply(x)).max() <= 1e-14 * np.linalg.norm(x)
    N = 16
    nn, nnn = oracle.bond_pairs(1, N, 4, 4)
    pairs = np.concatenate([nn, nnn])
    J = 1.0 + 0.1 * oracle.normal(2, len(pairs))
    D = 0.5 * J
    b16 = ed.Basis(envs(N), 1)
    hb = ed.Hamiltonian.from_bonds(envs(N), b16, pairs, J, D)
    hb.build_diag()
    hb.build_off_diag()
    Mb = Model(1, N, 4, 4, 1, bonds=pairs, Jb=J, Db=D)
    Mb.build(3)
    x = oracle.start_vector(4, b16.size)
    assert np.abs(hb.apply(x).cpu().numpy() - Mb.apply(x)).max() <= 1e-14 * np.linalg.norm(x)


def test_hv_nonfinite_input(ed, envs):
    env, b, h, M = make_pair(ed, envs, 0, 12, 1, 12, 0, 1.0, 1.0, 0.0, 0.0)
    x = oracle.start_vector(1, b.size)
    x[100] = np.nan
    for acc in ('exact', 'fixed64', 'fp64'):
        h.set_accumulation(acc)
        y = h.apply(x).cpu().numpy()
        assert np.isnan(y[100])
        cols = M.scipy()[:, 100].nonzero()[0]
        assert np.all(np.isnan(y[cols]))


@pytest.mark.parametrize('case', [
    (0, 16, 1, 16, 0, 1.0, 1.0, 0.3, 0.3),
    (1, 20, 4, 5, 0, 1.0, 1.0, 0.5, 0.5),
    (1, 24, 4, 6, 1, 1.0, 0.7, 0.55, 0.55),
])
def test_hv_real_input(ed, envs, case):
    """Real input (imaginary parts exactly zero): the fixed-point path keeps
    real parts only.  Within 1e-14 * ||x||_2 of the oracle, imaginary output
    exactly zero, and non-finite entries reach exactly the rows that gather
    them (the allocation-free kernel, which always gathers (re, im)
    pairs, is compared bit for bit in test_zz_no_alloc.py)."""
    ltype, N, lx, ly, mag, J1, D1, J2, D2 = case
    env, b, h, M = make_pair(ed, envs, ltype, N, lx, ly, mag, J1, D1, J2, D2)
    x = oracle.start_vector(6, b.size).real.astype(np.complex128)
    y = h.apply(x).cpu().numpy()
    assert np.abs(y - M.apply(x)).max() <= 1e-14 * np.linalg.norm(x)
    assert np.all(y.imag == 0.0)
    x[7] = np.inf
    y = h.apply(x).cpu().numpy()
    cols = set(M.scipy()[:, 7].nonzero()[0]) | {7}
    bad = set(np.nonzero(~np.isfinite(y.real))[0])
    assert bad == cols


@pytest.mark.parametrize('case', [
    (1, 20, 4, 5, 0, 1.0, 1.0, 0.5, 0.5),
    (1, 24, 4, 6, 1, 1.0, 0.7, 0.55, 0.55),
])
def test_hv_real_storage(ed, envs, case):
    """Real storage (float64 vectors, the solver's real mode): every launch
    variant gives the real part of the complex-storage H.v bit for bit, and a
    non-finite entry reaches exactly the rows that gather it (the checked
    path of each kernel).  The 4x6 case is above the autotuner's size
    threshold, so 'auto' times the variants there."""
    ltype, N, lx, ly, mag, J1, D1, J2, D2 = case
    env, b, h, M = make_pair(ed, envs, ltype, N, lx, ly, mag, J1, D1, J2, D2)
    xr = oracle.start_vector(9, b.size).real.copy()
    ref = h.apply(xr.astype(np.complex128)).cpu().numpy().real
    assert np.abs(ref - M.apply(xr.astype(np.complex128)).real).max() <= 1e-14 * np.linalg.norm(xr)
    xbad = xr.copy()
    xbad[7] = np.nan
    cols = set(M.scipy()[:, 7].nonzero()[0]) | {7}
    for v in ('auto', 'u4-b6', 'u4-b4', 'u8-b4', 'u8-b1', 'jit', 'jit-b4', 'jit-b3', 'jit-w3', 'jit-w4'):
        h.set_hv_variant(v)
        y = h.apply_real(xr).cpu().numpy()
        assert np.array_equal(y.view(np.uint64), ref.view(np.uint64)), v
        y = h.apply_real(xbad).cpu().numpy()
        assert set(np.nonzero(~np.isfinite(y))[0]) == cols, v
    h.set_hv_variant('auto')
    with pytest.raises(ed.InvalidArgument):
        h.apply_real(xr[:-1])


def test_hv_variants_bit_identical(ed, envs):
    """Every launch variant of the two-table H.v (static unroll / register
    budgets, and the kernel compiled at run time for this lattice's bonds)
    sums the same exact integers: results agree bit for bit, for complex and
    real inputs, and match the oracle within 1e-14 * ||x||_2.  Solves with the
    fused x^H y of each variant agree to 1e-12."""
    env, b, h, M = make_pair(ed, envs, 1, 20, 4, 5, 0, 1.0, 1.0, 0.5, 0.5)
    xc = oracle.start_vector(8, b.size)
    xr = xc.real.astype(np.complex128)
    ref = {}
    for v in ('u4-b6', 'u4-b4', 'u8-b4', 'u8-b1', 'jit', 'jit-b4', 'jit-b3', 'jit-w3', 'jit-w4'):
        h.set_hv_variant(v)
        for name, x in (('complex', xc), ('real', xr)):
            y = h.apply(x).cpu().numpy()
            if name not in ref:
                ref[name] = y
                assert np.abs(y - M.apply(x)).max() <= 1e-14 * np.linalg.norm(x)
            assert np.array_equal(y.view(np.uint64), ref[name].view(np.uint64)), (v, name)
        eps = ed.Solver.SolverInit(h, 3, 16)
        ed.Solver.EPSSetTolerances(eps, 1e-11)
        ed.Solver.solve(env, eps)
        ev = [ed.Solver.eigenvalue(eps, i)[0] for i in range(3)]
        ed.Solver.SolverClean(eps)
        if 'ev' not in ref:
            ref['ev'] = ev
        assert np.allclose(ev, ref['ev'], rtol=1e-12, atol=0), (v, ev, ref['ev'])
        assert h.hv_variant(False) == v and h.hv_variant(True) == v
    h.set_hv_variant('auto')
    with pytest.raises(ValueError):
        h.set_hv_variant('no-such-variant')


def test_hv_edge_cases(ed, envs):
    # one-state sector, all-up: H is the 1x1 diagonal
    env, b, h, M = make_pair(ed, envs, 0, 8, 1, 8, 4, 1.0, 1.0, 0.0, 0.0)
    assert b.size == 1
    y = h.apply(np.array([1.0 + 2.0j])).cpu().numpy()
    assert np.allclose(y, M.apply(np.array([1.0 + 2.0j])), rtol=0, atol=1e-15)
    # no couplings at all: zero operator
    env, b, h, M = make_pair(ed, envs, 0, 10, 1, 10, 0, 0.0, 0.0, 0.0, 0.0)
    x = oracle.start_vector(1, b.size)
    assert np.abs(h.apply(x).cpu().numpy()).max() == 0.0
    # N = 2 chain: nnn bonds are self bonds (i == j) and never couple
    env, b, h, M = make_pair(ed, envs, 0, 2, 1, 2, 0, 1.0, 1.0, 1.0, 1.0)
    x = oracle.start_vector(2, b.size)
    assert np.abs(h.apply(x).cpu().numpy() - M.apply(x)).max() <= 1e-15
    _csr_equal(h, M)


# ---------------------------------------------------------------------------
# eigensolver
# ---------------------------------------------------------------------------
def _match_levels(ev, expected, tol):
    idx = [i for i, _, _ in expected]
    vals = np.array([v for _, v, _ in expected])
    ev = np.asarray(ev)
    if len(ev) > max(idx) and np.all(np.abs(ev[idx] - vals) <= tol * np.maximum(1.0, np.abs(vals))):
        return True
    distinct = [ev[0]]
    for e in ev[1:]:
        if abs(e - distinct[-1]) > 1e-8:
            distinct.append(e)
    distinct = np.array(distinct)
    return len(distinct) > max(idx) and bool(
        np.all(np.abs(distinct[idx] - vals) <= tol * np.maximum(1.0, np.abs(vals))))


def solve(ed, env, h, nev, tol=1e-12, ncv=None, restart=None):
    eps = ed.Solver.SolverInit(h, nev, ncv if ncv else max(2 * nev, nev + 15))
    ed.Solver.EPSSetTolerances(eps, tol, 0)
    if restart:
        eps.set_restart_arithmetic(restart)
    nconv = ed.Solver.solve(env, eps)
    st = eps.stats()
    evals, errs = [], []
    for i in range(st['nreported']):
        e, err = ed.Solver.eigenvalue(eps, i)
        evals.append(e)
        errs.append(err)
    return eps, nconv, np.array(evals), np.array(errs)


def test_real_storage_matches_complex_path(ed, envs):
    """The seeded (real) start vector runs the real-storage solver; a complex
    start vector runs the complex path.  Same eigenvalues (1e-10 relative),
    residuals within tol, and the real-storage eigenvectors come back as
    complex128 with exactly zero imaginary parts."""
    hi = oracle.rd_hi(4, 16, -1.0, 1.0)  # fields lift the lattice degeneracies
    env, b, h, M = make_pair(ed, envs, 0, 16, 1, 16, 0, 1.0, 1.0, 0.3, 0.3,
                             ('build_diag', 'build_off_diag', 'build_disorder'), hi)
    eps, nconv, ev_r, err_r = solve(ed, env, h, 4, tol=1e-11, ncv=16)
    ev_r, err_r = ev_r[:4], err_r[:4]
    vecs = [ed.Solver.solution(eps, i)[1].cpu().numpy() for i in range(4)]
    host = ed.Solver.solution_host(eps, 0)
    ed.Solver.SolverClean(eps)
    for v in vecs:
        assert np.all(v.imag == 0.0)
    assert np.array_equal(host.view(np.uint64), vecs[0].view(np.uint64))
    eps = ed.Solver.SolverInit(h, 4, 16)
    ed.Solver.EPSSetTolerances(eps, 1e-11)
    eps.set_initial_vector(oracle.start_vector(3, b.size))
    ed.Solver.solve(env, eps)
    ev_c = [ed.Solver.eigenvalue(eps, i)[0] for i in range(4)]
    ed.Solver.SolverClean(eps)
    assert np.allclose(ev_r, ev_c, rtol=1e-10, atol=0), (ev_r, ev_c)
    w = np.linalg.eigvalsh(M.dense())
    assert np.allclose(ev_r, w[:4], rtol=1e-10, atol=0)
    assert max(err_r) <= 1e-11


@pytest.mark.parametrize('case', [(18, 7), (8, 4), (16, 0)])
def test_host_eigenvector_real_storage(ed, envs, case):
    """solution_host of a real-storage solve (staged in halves through a spare
    basis column and the work vector) equals the device eigenvector bit for
    bit, for an odd dimension (C(18,16) = 153: a third chunk reuses a stage),
    the one-state sector and an even one."""
    N, mag = case
    env, b, h, M = make_pair(ed, envs, 0, N, 1, N, mag, 1.0, 1.0, 0.3, 0.3)
    nev = 1 if b.size == 1 else 2
    eps, nconv, ev, errs = solve(ed, env, h, nev, tol=1e-10, ncv=min(16, b.size))
    assert nconv >= nev
    for i in range(nev):
        dev = ed.Solver.solution(eps, i)[1].cpu().numpy()
        host = ed.Solver.solution_host(eps, i)
        assert np.array_equal(host.view(np.uint64), dev.view(np.uint64)), (case, i)
        assert np.all(host.imag == 0.0)
    ed.Solver.SolverClean(eps)


def test_restart_pair_arithmetic(ed, envs, golden):
    """Float-pair products in the restart combination (forced here; opt-in,
    the default keeps FP64): every golden solver case at 1e-12 as
    with FP64 products, and on the 4x6 lattice (2.7M states) the same lowest
    levels as the FP64 products at 1e-12 relative, residuals within tol and
    orthonormal Ritz vectors."""
    for rec in golden['solver']:
        env, b, h, M = make_pair(ed, envs, rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['J1'],
                                 rec['D1'], rec['J2'], rec['D2'], rec['calls'])
        want = max(i for i, _, _ in rec['expected']) + 1
        eps, nconv, ev, errs = solve(ed, env, h, max(want, rec['nev']), restart='pair')
        assert nconv >= want, rec['name']
        assert _match_levels(ev, rec['expected'], 1e-12), (rec['name'], ev, rec['expected'])
        assert np.all(errs[:want] <= 1e-8), (rec['name'], errs)
        ed.Solver.SolverClean(eps)
    env, b, h, M = make_pair(ed, envs, 1, 24, 4, 6, 0, 1.0, 1.0, 0.55, 0.55)
    out = {}
    for gs in ('fp64', 'pair'):
        eps, nconv, ev, errs = solve(ed, env, h, 4, tol=1e-10, ncv=16, restart=gs)
        assert nconv >= 4 and np.all(errs[:4] <= 1e-10), (gs, errs)
        X = np.stack([ed.Solver.solution(eps, i)[1].cpu().numpy().real for i in range(4)])
        ed.Solver.SolverClean(eps)
        assert np.abs(X @ X.T - np.eye(4)).max() <= 1e-12, gs
        out[gs] = ev[:4]
    assert np.allclose(out['pair'], out['fp64'], rtol=1e-12, atol=0), out
    eps = ed.Solver.SolverInit(h, 2, 16)
    with pytest.raises(ed.InvalidArgument):
        eps.set_restart_arithmetic('fp16')
    ed.Solver.SolverClean(eps)


def test_golden_eigenvalues(ed, envs, golden):
    for rec in golden['solver']:
        env, b, h, M = make_pair(ed, envs, rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['J1'],
                                 rec['D1'], rec['J2'], rec['D2'], rec['calls'])
        want = max(i for i, _, _ in rec['expected']) + 1
        eps, nconv, ev, errs = solve(ed, env, h, max(want, rec['nev']))
        assert nconv >= want, rec['name']
        assert _match_levels(ev, rec['expected'], 1e-12), (rec['name'], ev, rec['expected'])
        assert np.all(errs[:want] <= 1e-8), (rec['name'], errs)
        ed.Solver.SolverClean(eps)


def test_eigenvalues_vs_dense(ed, envs):
    # 4x3 copy of the 4x5 J1-J2 workload: FP64 dense diagonalisation oracle
    env, b, h, M = make_pair(ed, envs, 1, 12, 4, 3, 0, 1.0, 1.0, 0.5, 0.5)
    ev_dense = np.linalg.eigvalsh(M.dense())
    eps, nconv, ev, errs = solve(ed, env, h, 10, tol=1e-10)
    assert nconv >= 10
    assert np.all(errs[:10] <= 1e-9)
    _check_krylov_levels(ev[:10], ev_dense, 1e-10)


def _check_krylov_levels(ev, ev_dense, rtol):
    """A single-vector Krylov method can miss copies of a degenerate level
    (as SLEPc's can): every returned value must be an eigenvalue, counted at
    most as often as it occurs, and every distinct level below the largest
    returned value must be present."""
    ev = np.sort(ev)
    tol = rtol * np.abs(ev_dense).max()
    used = np.zeros(len(ev_dense), bool)
    for e in ev:
        k = np.where(~used & (np.abs(ev_dense - e) <= tol))[0]
        assert len(k), (e, ev_dense[:len(ev) + 4])
        used[k[0]] = True
    below = ev_dense[ev_dense <= ev[-1] + tol]
    levels = [below[0]] + [x for a, x in zip(below[:-1], below[1:]) if x - a > 1e-8]
    for lv in levels:
        assert np.any(np.abs(ev - lv) <= tol), ('missing level', lv)


def test_solver_deterministic(ed, envs):
    env, b, h, M = make_pair(ed, envs, 1, 16, 4, 4, 0, 1.0, 1.0, 0.5, 0.5)
    _, _, ev1, _ = solve(ed, env, h, 2)
    _, _, ev2, _ = solve(ed, env, h, 2)
    assert np.array_equal(ev1, ev2)


def test_solver_errors(ed, envs):
    env, b, h, M = make_pair(ed, envs, 0, 8, 1, 8, 0, 1.0, 1.0, 0.0, 0.0)
    eps = ed.Solver.SolverInit(h, 1)
    with pytest.raises(ed.EDError):
        ed.Solver.eigenvalue(eps, 0)  # before solve
    ed.Solver.solve(env, eps)
    with pytest.raises(ValueError):
        ed.Solver.eigenvalue(eps, 99)


# ---------------------------------------------------------------------------
# correlations, magnetisation, DSF
# ---------------------------------------------------------------------------
def test_golden_correlations(ed, envs, golden):
    cls = {'SzSz': ed.SzSz, 'SpSm': ed.SpSm}
    for rec in golden['correlation']:
        env, b, h, M = make_pair(ed, envs, rec['ltype'], rec['N'], rec['lx'], rec['ly'], rec['mag'], rec['J1'],
                                 rec['D1'], rec['J2'], rec['D2'])
        eps, nconv, ev, errs = solve(ed, env, h, 1)
        assert abs(ev[0] - rec['E0']) <= 1e-12 * abs(rec['E0'])
        _, psi, _ = ed.Solver.solution(eps, 0)
        corr = cls[rec['op']](env, b)
        pairs = [(i, j) for i, j, _, _ in rec['pairs']]
        vals = corr.ExpectValPairs(pairs, psi)
        for (i, j, v, tol), got in zip(rec['pairs'], vals):
            assert abs(got.real - v) <= tol, (rec['name'], i, j, got, v)
        # single-pair entry point agrees
        assert abs(corr.ExpectVal(env, pairs[0][0], pairs[0][1], psi) - vals[0]) <= 1e-15


def test_correlations_vs_oracle(ed, envs):
    env, b, h, M = make_pair(ed, envs, 1, 12, 4, 3, 0, 1.0, 1.0, 0.5, 0.5)
    psi = oracle.start_vector(21, b.size)
    psi /= np.linalg.norm(psi)
    for op, cls in ((0, ed.SzSz), (1, ed.SpSm), (2, ed.SmSp), (3, ed.SiSj)):
        got = cls(env, b).AllPairs(psi)
        for i in range(12):
            for j in range(12):
                ref = M.expect(op, i, j, psi)
                assert abs(got[i, j] - ref) <= 1e-14, (op, i, j, got[i, j], ref)


@pytest.mark.parametrize('ltype,N,lx,ly,mag', [(1, 12, 4, 3, 0), (0, 14, 14, 1, 1), (1, 16, 4, 4, 2)])
def test_correlations_real_state_vs_oracle(ed, envs, ltype, N, lx, ly, mag):
    """A real state (the solver's eigenvectors are real): S^z S^z and S.S run
    a kernel of their own (compact real copy of the state, the flipped state's
    rank from the row's own), SpSm / SmSp the general one.  All four
    operators, all N^2 pairs, against the oracle at 1e-14; pairs inside the
    low half of the rank table, inside the high half, and across."""
    env, b, h, M = make_pair(ed, envs, ltype, N, lx, ly, mag, 1.0, 1.0, 0.5, 0.5)
    psi = oracle.start_vector(22 + N, b.size).real.copy()
    psi /= np.linalg.norm(psi)
    for op, cls in ((0, ed.SzSz), (1, ed.SpSm), (2, ed.SmSp), (3, ed.SiSj)):
        got = cls(env, b).AllPairs(psi)
        assert np.abs(got - got.T.conj()).max() == 0.0, op
        for i in range(N):
            for j in range(N):
                ref = M.expect(op, i, j, psi)
                assert abs(got[i, j] - ref) <= 1e-14, (op, i, j, got[i, j], ref)


def test_correlations_wide_range_state(ed, envs):
    """One large amplitude and 12,869 of size 0.8 2^-30 (random signs): the
    S^z S^z sums of the real-state kernel are exact integer sums of psi_r^2 at
    a scale fixed by their total, so the tiny weights must not be rounded
    away (at 2^-59 resolution each would lose about 2^-60, 1e-14 in all).
    Against the oracle at 1e-15."""
    env, b, h, M = make_pair(ed, envs, 1, 16, 4, 4, 0, 1.0, 1.0, 0.5, 0.5)
    rng = np.random.default_rng(11)
    psi = np.where(rng.random(b.size) < 0.5, -1.0, 1.0) * (0.8 * 2.0 ** -30)
    psi[0] = 1.0
    for op, cls in ((0, ed.SzSz), (3, ed.SiSj)):
        got = cls(env, b).AllPairs(psi)
        for i in range(16):
            for j in range(16):
                ref = M.expect(op, i, j, psi)
                assert abs(got[i, j] - ref) <= 1e-15, (op, i, j, got[i, j], ref)


@pytest.mark.parametrize('N,lx,ly,mag,wide', [(12, 4, 3, 0, False), (16, 4, 4, 1, True)])
def test_szsz_real_state_bit_exact_vs_model(ed, envs, N, lx, ly, mag, wide):
    """The S^z S^z sums of a real state (exact 128-bit integer sums of the
    FP64 weights psi_r^2, rounded once) bit for bit against the host
    restatement tests/zz_model.py, for every pair."""
    import zz_model
    env = envs(N)
    b = ed.Basis(env, mag)
    states = zz_model.basis_states(N, N // 2 + mag)
    assert len(states) == b.size
    rng = np.random.default_rng(N + mag)
    psi = rng.standard_normal(b.size)
    if wide:
        psi *= np.exp2(-rng.integers(0, 40, b.size))
        psi[0] = 1.2
    else:
        psi *= np.sqrt(1.5) / np.linalg.norm(psi)  # sum of weights away from a power of two
    got = ed.SzSz(env, b).AllPairs(psi).real
    pairs = [(i, j) for i in range(N) for j in range(i, N)]
    want = zz_model.szsz(states, psi, pairs)
    for (i, j), w in zip(pairs, want):
        assert got[i, j].view(np.uint64) == np.float64(w).view(np.uint64), (i, j, got[i, j], w)
        assert got[j, i] == got[i, j]


def test_correlations_nonfinite_state(ed, envs):
    """A real state with a NaN entry: S.S and S^z S^z fall back to the general
    kernel (their fixed-point sums need a finite norm) and every pair is NaN,
    as in FP64."""
    env, b, h, M = make_pair(ed, envs, 1, 12, 4, 3, 0, 1.0, 1.0, 0.5, 0.5)
    psi = oracle.start_vector(7, b.size).real.copy()
    psi[17] = np.nan
    for cls in (ed.SzSz, ed.SiSj):
        C = cls(env, b).AllPairs(psi)
        assert np.isnan(C.real).all(), cls


def test_sublattice_magnetisation(ed, envs):
    env, b, h, M = make_pair(ed, envs, 1, 16, 4, 4, 0, 1.0, 1.0, 0.0, 0.0)
    eps, nconv, ev, errs = solve(ed, env, h, 1)
    _, psi, _ = ed.Solver.solution(eps, 0)
    lat = ed.square2D(env, 4, 4)
    af, st = ed.AF(lat, 2), ed.Striped(lat, 4)
    assert af.sublat == oracle.sublattice_af(1, 16, 4, 4)
    assert st.sublat == oracle.sublattice_striped(1, 16, 4, 4)
    psi_h = psi.cpu().numpy()
    m_af = ed.Phys.SquaredSubLattMagAF(env, b, af, psi)
    m_st = ed.Phys.SquaredSubLattMagSTR(env, b, st, psi)
    assert abs(m_af - oracle.squared_sublatt_mag_af(M, af.sublat, psi_h)) <= 1e-12
    assert abs(m_st - oracle.squared_sublatt_mag_str(M, st.sublat, psi_h)) <= 1e-12


def test_dsf_coefficients_vs_oracle(ed, envs):
    import torch
    N = 10
    env = envs(N)
    for op in (0, 1):
        M0 = Model(0, N, 1, N, 0, 1.0, 1.0, 0.2, 0.2)
        M0.build(3)
        M1 = M0 if op == 0 else Model(0, N, 1, N, 1, 1.0, 1.0, 0.2, 0.2)
        if op == 1:
            M1.build(3)
        w, V = np.linalg.eigh(M1.dense())
        psi = oracle.start_vector(5, M0.dim)
        psi /= np.linalg.norm(psi)
        vecs = np.ascontiguousarray(V[:, :6].T.astype(np.complex128) * np.exp(0.3j))
        b0 = ed.Basis(env, 0)
        b1 = b0 if op == 0 else ed.Basis(env, 1)
        c = ed.Phys.dsf_coefficients(env, b0, b1, op, psi, torch.from_numpy(vecs))
        for i in range(N):
            rhs = M0.sqz(i, psi) if op == 0 else M0.sqp(M1, i, psi)
            for n in range(6):
                ref = oracle.vecdot(rhs, vecs[n])
                assert abs(c[i, n] - ref) <= 1e-14, (op, i, n, c[i, n], ref)


def test_golden_dsf_pipeline(ed, envs, golden, tmp_path):
    for rec in golden['dsf']:
        N = rec['N']
        env = envs(N)
        b0 = ed.Basis(env, rec['mag0'])
        b1 = b0 if rec['mag1'] == rec['mag0'] else ed.Basis(env, rec['mag1'])
        lat = ed.chain1D(env)
        h0 = ed.Hamiltonian(env, b0, lat, rec['J1'], rec['D1'], rec['J2'], rec['D2'])
        h0.build_diag(env)
        h0.build_off_diag(env)
        h1 = h0
        if b1 is not b0:
            h1 = ed.Hamiltonian(env, b1, lat, rec['J1'], rec['D1'], rec['J2'], rec['D2'])
            h1.build_diag(env)
            h1.build_off_diag(env)
        eps, nconv, ev, errs = solve(ed, env, h0, 1)
        gs, psi, _ = ed.Solver.solution(eps, 0)
        assert abs(gs - rec['GS']) <= 1e-12
        data = ed.DSF_data(b0=b0, b1=b1, lat=lat, h0=h0, h1=h1, nev=rec['nev'], path=str(tmp_path))
        ed.Solver.options = {'eps_tol': 1e-12}
        try:
            dE, c = ed.Phys.DynStructFactor(env, data, gs, psi, 0, 'Sqz' if rec['op'] == 'Sqz' else 'Sqp')
        finally:
            ed.Solver.options = {}
        ref_E = np.array([row[0] for row in rec['spins'][0]])
        assert np.allclose(dE, ref_E, atol=1e-10), (dE, ref_E)
        # file layout: header lines and one block per spin
        lines = open(tmp_path / 'dsf_d0.dat').read().split('\n')
        assert lines[1] == '# nspins:   %d  ' % N
        assert lines[2] == '#    nev:   %d  ' % rec['nev']
        assert sum(1 for l in lines if l.startswith('# spin:')) == N
        # sum rule per site: sum_n |c_{i,n}|^2 <= <0|S_i^dag S_i|0> (1/4 for S^z, <= 1 for S^+)
        bound = 0.25 if rec['op'] == 'Sqz' else 1.0
        assert np.all(np.sum(np.abs(c) ** 2, axis=1) <= bound + 1e-12)


def test_dsf_spectrum_vs_oracle(ed, envs):
    """Device S(q, w) (Lorentzian broadening of the DSF weights, the
    post-processing notebook's cells 11-15) against the oracle's restatement,
    1e-12 of the largest value; realisations accumulate in place."""
    N, lx, ly, nev = 16, 4, 4, 40
    env = envs(N)
    rng = np.random.default_rng(11)
    qs = oracle.q_grid(N, lx, ly)
    pos = np.array([(i // ly, i % ly) for i in range(N)], dtype=np.float64)
    spectra = []
    S = None
    for rep in range(3):
        c = rng.standard_normal((N, nev)) + 1j * rng.standard_normal((N, nev))
        dE = np.sort(rng.uniform(0.0, 4.5, nev))
        ref = oracle.dsf_spectrum(c, dE, pos, qs, nw=5001)
        one = ed.Phys.dsf_spectrum(env, c, dE, pos, qs, nw=5001).cpu().numpy()
        assert np.abs(one - ref).max() <= 1e-12 * np.abs(ref).max()
        S = ed.Phys.dsf_spectrum(env, c, dE, pos, qs, nw=5001, out=S)
        spectra.append(ref)
    avg = 2 * np.pi * S.cpu().numpy() / 3
    ref_avg = oracle.dsf_average(spectra)
    assert np.abs(avg - ref_avg).max() <= 1e-12 * np.abs(ref_avg).max()
    with pytest.raises(ValueError):
        ed.Phys.dsf_spectrum(env, c, dE[:-1], pos, qs)


def test_dsf_spectrum_sum_rule(ed, envs):
    """Full Sz=0 spectrum of a chain (N=8), coefficients from the device:
    the notebooks' sum rule sum_{q,w} S dw / 2 pi = 1/4 (window widened to
    [-40, 40] so the Lorentzian tails stay inside; missing weight < 2e-3),
    and the notebook window [0, 5] equal to the oracle's value."""
    import torch
    N = 8
    env = envs(N)
    M = Model(0, N, 1, N, 0, 1.0, 1.0, 0.0, 0.0)
    M.build(3)
    w, V = np.linalg.eigh(M.dense())
    b = ed.Basis(env, 0)
    vecs = np.ascontiguousarray(V.T.astype(np.complex128))
    c = ed.Phys.dsf_coefficients(env, b, b, 0, vecs[0], torch.from_numpy(vecs))
    dE = w - w[0]
    qs = oracle.q_grid(N, 1, N)
    pos = np.array([(0, i) for i in range(N)], dtype=np.float64)
    wide = ed.Phys.dsf_spectrum(env, c, dE, pos, qs, nw=160001, w_min=-40.0, w_max=40.0)
    assert abs(ed.Phys.dsf_sum_rule(2 * np.pi * wide, -40.0, 40.0) - 0.25) < 2e-3
    S = 2 * np.pi * ed.Phys.dsf_spectrum(env, c, dE, pos, qs, nw=5001).cpu().numpy()
    ref = oracle.dsf_average([oracle.dsf_spectrum(c, dE, pos, qs)])
    assert abs(ed.Phys.dsf_sum_rule(S) - oracle.dsf_sum_rule(ref)) <= 1e-12


@pytest.mark.parametrize('case', [(1, 16, 4, 4, 1), (1, 24, 4, 6, 0), (0, 12, 1, 12, 0)])
def test_hv_per_bond_fixed_point(ed, envs, case):
    """Per-bond couplings (J_b = base_b (1 + 0.1 z_b), D_b = J_b, fields):
    the run-time compiled fixed-point H.v, each bond's J_b / 2 a 64-bit
    immediate and each row's sum exact in 128 bits, matches the oracle's
    explicit matrix within 1e-14 * ||x||_2 for complex and real input, in
    real storage (plain and fused with x^T y), with every register budget
    bit-identical; a static variant is refused for a per-bond operator."""
    ltype, N, lx, ly, mag = case
    nn, nnn = oracle.bond_pairs(ltype, N, lx, ly)
    pairs = np.concatenate([nn, nnn])
    z = oracle.normal(91, len(pairs))
    J = np.where(np.arange(len(pairs)) < len(nn), 1.0, 0.5) * (1 + 0.1 * z)
    D = J.copy()
    hi = oracle.rd_hi(92, N, -0.5, 0.5)
    env = envs(N)
    b = ed.Basis(env, mag)
    h = ed.Hamiltonian.from_bonds(env, b, pairs, J, D)
    h.build_diag(env)
    h.build_off_diag(env)
    h.build_disorder(env, hi)
    M = Model(0, N, 1, N, mag, bonds=pairs, Jb=J, Db=D)
    M.build(7, hi)
    x = oracle.start_vector(93, b.size)
    tol = 1e-14 * np.linalg.norm(x)
    assert np.abs(h.apply(x).cpu().numpy() - M.apply(x)).max() <= tol
    xr = x.real.copy()
    ref = M.apply(xr.astype(np.complex128)).real
    first = None
    for v in ('jit', 'jit-b4', 'jit-b3', 'jit-w3', 'jit-w4'):
        h.set_hv_variant(v)
        y = h.apply_real(xr).cpu().numpy()
        assert np.abs(y - ref).max() <= 1e-14 * np.linalg.norm(xr), v
        y2, xy, yy = h.apply_real_dot(xr)
        assert np.array_equal(y2.cpu().numpy().view(np.uint64), y.view(np.uint64)), v
        assert abs(xy - xr @ y) <= 1e-12 * abs(xy) and abs(yy - y @ y) <= 1e-12 * yy
        if first is None:
            first = y
        assert np.array_equal(y.view(np.uint64), first.view(np.uint64)), v
    with pytest.raises(ed.EDError):
        h.set_hv_variant('u4-b6')
    h.set_hv_variant('auto')
