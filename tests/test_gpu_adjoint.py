"""Adjoint gradients (Adjoint / ed_expect_mixed / ed_apply_term /
ed_grad_energy / ed_minres) against dense numpy algebra on the oracle's basis
and Hamiltonian, and against central finite differences.

Workloads follow the per-bond disorder case: J1-J2 couplings
J_b = base_b (1 + 0.1 z_b), z_b ~ N(0, 1), D_b = J_b, fields h_i ~ U[-0.5, 0.5].

Tolerances: term application and mixed expectations within 1e-14 * ||.||
(products by 0.25 / 0.5 are exact); Hellmann-Feynman gradients within 1e-9 of
the dense eigenvector's expectations; finite differences (step 1e-4, error
O(step^2)) within 1e-6; MINRES solutions within 1e-9 relative.
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


@pytest.fixture(scope='module')
def envs(ed):
    cache = {}

    def get(n):
        if n not in cache:
            cache[n] = ed.Environment(nspins=n)
        return cache[n]
    return get


def disordered(ltype, N, lx, ly, seed, J2=0.55):
    nn, nnn = oracle.bond_pairs(ltype, N, lx, ly)
    pairs = np.concatenate([nn, nnn])
    z = oracle.normal(seed, len(pairs))
    J = np.where(np.arange(len(pairs)) < len(nn), 1.0, J2) * (1 + 0.1 * z)
    D = J.copy()
    hi = oracle.rd_hi(seed + 1, N, -0.5, 0.5)
    return pairs, J, D, hi


def dense_model(N, mag, pairs, J, D, hi):
    M = Model(0, N, 1, N, mag, bonds=pairs, Jb=J, Db=D)
    M.build(7, hi)
    return M


def term_matrix(states, kind, i, j):
    """Dense O for one term on the sector basis (rows/cols = basis index)."""
    idx = {int(s): r for r, s in enumerate(states)}
    n = len(states)
    O = np.zeros((n, n))
    for r, s in enumerate(states):
        s = int(s)
        a, b = (s >> i) & 1, (s >> j) & 1
        if kind == 2:
            O[r, r] += 0.5 if a else -0.5
            continue
        if kind in (1, 3):
            O[r, r] += -0.25 if a != b else 0.25
        if kind in (0, 3):
            if i == j:
                O[r, r] += 0.5
            elif a != b:
                O[idx[s ^ ((1 << i) | (1 << j))], r] += 0.5
    return O


TERMS = [(0, 0, 3), (1, 0, 3), (2, 4, 4), (3, 2, 7), (0, 5, 5), (3, 6, 6), (1, 9, 1), (0, 8, 2), (2, 0, 0)]


def test_apply_term_and_mixed_match_dense(ed, envs):
    N, mag = 10, 0
    env = envs(N)
    b = ed.Basis(env, mag)
    M = Model(0, N, 1, N, mag)
    states = M.states()
    assert np.array_equal(states, b.int_basis.astype(np.uint64))
    rng = np.random.default_rng(3)
    psi = rng.standard_normal(b.size) + 1j * rng.standard_normal(b.size)
    lam = rng.standard_normal(b.size) + 1j * rng.standard_normal(b.size)
    ref_mixed = []
    for kind, i, j in TERMS:
        O = term_matrix(states, kind, i, j)
        y = ed.Adjoint.apply_term(b, kind, i, j, psi).cpu().numpy()
        assert np.abs(y - O @ psi).max() <= 1e-14 * np.linalg.norm(psi), (kind, i, j)
        ref_mixed.append(np.vdot(lam, O @ psi))
    got = ed.Adjoint.expect_mixed(b, TERMS, lam, psi)
    scale = np.linalg.norm(lam) * np.linalg.norm(psi)
    assert np.abs(got - np.array(ref_mixed)).max() <= 1e-13 * scale


def test_apply_term_rejects_bad_input(ed, envs):
    env = envs(8)
    b = ed.Basis(env, 0)
    psi = np.ones(b.size, dtype=np.complex128)
    with pytest.raises(ValueError):
        ed.Adjoint.apply_term(b, 7, 0, 1, psi)
    with pytest.raises(ValueError):
        ed.Adjoint.apply_term(b, 0, 0, 8, psi)
    with pytest.raises(ValueError):
        ed.Adjoint.expect_mixed(b, [(0, -1, 2)], psi, psi)


@pytest.mark.parametrize('case', [(0, 12, 1, 12, 0, 11), (1, 16, 4, 4, 0, 21)])
def test_energy_gradient_hellmann_feynman(ed, envs, case):
    ltype, N, lx, ly, mag, seed = case
    pairs, J, D, hi = disordered(ltype, N, lx, ly, seed)
    env = envs(N)
    b = ed.Basis(env, mag)
    h = ed.Hamiltonian.from_bonds(env, b, pairs, J, D)
    h.build_diag(env)
    h.build_off_diag(env)
    h.build_disorder(env, hi)
    eps = ed.Solver.SolverInit(h, 2, 20)
    ed.Solver.EPSSetTolerances(eps, 1e-12)
    ed.Solver.solve(env, eps)
    e0, v, _ = ed.Solver.solution(eps, 0)
    dJ, dD, dh = ed.Adjoint.energy_gradient(b, pairs, v)
    # the same expectations from the oracle's eigenvector and correlation code
    M = dense_model(N, mag, pairs, J, D, hi)
    res = M.eps_solve(nev=2, ncv=20, tol=1e-12)
    assert abs(res['evals'][0] - e0) <= 1e-10 * abs(e0)
    w = res['evecs'][0]
    w = w / np.linalg.norm(w)
    for q, (i, j) in enumerate(pairs):
        xy = 0.5 * (M.expect(1, int(i), int(j), w) + M.expect(2, int(i), int(j), w)).real
        zz = M.expect(0, int(i), int(j), w).real
        assert abs(dJ[q] - xy) <= 1e-9, (q, dJ[q], xy)
        assert abs(dD[q] - zz) <= 1e-9, (q, dD[q], zz)
    # sum rule: E0 = sum_b J_b <XY_b> + D_b <ZZ_b> + sum_i h_i <S^z_i>
    assert abs(J @ dJ + D @ dD + hi @ dh - e0) <= 1e-9 * abs(e0)
    ed.Solver.SolverClean(eps)


def test_energy_gradient_finite_differences(ed, envs):
    N, mag = 12, 0
    pairs, J, D, hi = disordered(0, N, 1, N, 31, J2=0.3)
    env = envs(N)
    b = ed.Basis(env, mag)
    h = ed.Hamiltonian.from_bonds(env, b, pairs, J, D)
    h.build_diag(env)
    h.build_off_diag(env)
    h.build_disorder(env, hi)
    eps = ed.Solver.SolverInit(h, 1, 16)
    ed.Solver.EPSSetTolerances(eps, 1e-12)
    ed.Solver.solve(env, eps)
    e0, v, _ = ed.Solver.solution(eps, 0)
    dJ, dD, dh = ed.Adjoint.energy_gradient(b, pairs, v)

    def E(Jx, Dx, hx):
        return np.linalg.eigvalsh(dense_model(N, mag, pairs, Jx, Dx, hx).dense())[0]

    d = 1e-4
    for q in (0, 5, 13, 20):
        Jp, Jm = J.copy(), J.copy()
        Jp[q] += d
        Jm[q] -= d
        assert abs((E(Jp, D, hi) - E(Jm, D, hi)) / (2 * d) - dJ[q]) <= 1e-6
        Dp, Dm = D.copy(), D.copy()
        Dp[q] += d
        Dm[q] -= d
        assert abs((E(J, Dp, hi) - E(J, Dm, hi)) / (2 * d) - dD[q]) <= 1e-6
    for i in (0, 7):
        hp, hm = hi.copy(), hi.copy()
        hp[i] += d
        hm[i] -= d
        assert abs((E(J, D, hp) - E(J, D, hm)) / (2 * d) - dh[i]) <= 1e-6
    ed.Solver.SolverClean(eps)


def test_minres_definite_and_projected(ed, envs):
    N, mag = 12, 1
    pairs, J, D, hi = disordered(0, N, 1, N, 41)
    env = envs(N)
    b = ed.Basis(env, mag)
    h = ed.Hamiltonian.from_bonds(env, b, pairs, J, D)
    h.build_diag(env)
    h.build_off_diag(env)
    h.build_disorder(env, hi)
    H = dense_model(N, mag, pairs, J, D, hi).dense()
    w, U = np.linalg.eigh(H)
    rng = np.random.default_rng(5)
    rhs = rng.standard_normal(b.size) + 1j * rng.standard_normal(b.size)
    # definite shift below the spectrum
    sigma = w[0] - 0.7
    x, its, rel = ed.Adjoint.minres(h, sigma, rhs, tol=1e-13)
    xr = np.linalg.solve(H - sigma * np.eye(b.size), rhs)
    assert rel <= 1e-13 and its > 0
    assert np.linalg.norm(x.cpu().numpy() - xr) <= 1e-9 * np.linalg.norm(xr)
    # singular shift at E0, projected onto the complement of psi0
    psi0 = U[:, 0].astype(np.complex128)
    rhs_p = rhs - np.vdot(psi0, rhs) * psi0
    x, its, rel = ed.Adjoint.minres(h, w[0], rhs_p, q=psi0, tol=1e-13)
    x = x.cpu().numpy()
    Hp = H - w[0] * np.eye(b.size)
    xr = U[:, 1:] @ ((U[:, 1:].conj().T @ rhs_p) / (w[1:] - w[0]))
    assert abs(np.vdot(psi0, x)) <= 1e-10 * np.linalg.norm(x)
    assert np.linalg.norm(Hp @ x - rhs_p) <= 1e-10 * np.linalg.norm(rhs_p)
    assert np.linalg.norm(x - xr) <= 1e-9 * np.linalg.norm(xr)


def test_expectation_gradient_finite_differences(ed, envs):
    N, mag = 12, 0
    pairs, J, D, hi = disordered(0, N, 1, N, 51, J2=0.3)
    env = envs(N)
    b = ed.Basis(env, mag)
    h = ed.Hamiltonian.from_bonds(env, b, pairs, J, D)
    h.build_diag(env)
    h.build_off_diag(env)
    h.build_disorder(env, hi)
    eps = ed.Solver.SolverInit(h, 1, 16)
    ed.Solver.EPSSetTolerances(eps, 1e-13)
    ed.Solver.solve(env, eps)
    e0, v, _ = ed.Solver.solution(eps, 0)
    # staggered spin correlation from site 0: O = sum_j (-1)^j S_0 . S_j
    obs = [((-1.0) ** j, ed.Adjoint.SISJ, 0, j) for j in range(N)]
    val, dJ, dD, dh, info = ed.Adjoint.expectation_gradient(h, pairs, e0, v, obs, tol=1e-13)
    assert info['relres'] <= 1e-12
    states = Model(0, N, 1, N, mag).states()
    O = sum(c * term_matrix(states, k, i, j) for c, k, i, j in obs)

    def expval(Jx, Dx, hx):
        _, U = np.linalg.eigh(dense_model(N, mag, pairs, Jx, Dx, hx).dense())
        u = U[:, 0]
        return float(np.real(np.vdot(u, O @ u)))

    assert abs(val - expval(J, D, hi)) <= 1e-9
    d = 1e-4
    for q in (1, 8, 17):
        Jp, Jm = J.copy(), J.copy()
        Jp[q] += d
        Jm[q] -= d
        fd = (expval(Jp, D, hi) - expval(Jm, D, hi)) / (2 * d)
        assert abs(fd - dJ[q]) <= 1e-6 * max(1.0, abs(fd)), (q, fd, dJ[q])
        Dp, Dm = D.copy(), D.copy()
        Dp[q] += d
        Dm[q] -= d
        fd = (expval(J, Dp, hi) - expval(J, Dm, hi)) / (2 * d)
        assert abs(fd - dD[q]) <= 1e-6 * max(1.0, abs(fd)), (q, fd, dD[q])
    for i in (2, 9):
        hp, hm = hi.copy(), hi.copy()
        hp[i] += d
        hm[i] -= d
        fd = (expval(J, D, hp) - expval(J, D, hm)) / (2 * d)
        assert abs(fd - dh[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, dh[i])
    ed.Solver.SolverClean(eps)


def test_ground_state_energy_autograd(ed, envs):
    import torch
    N, mag = 12, 0
    pairs, J, D, hi = disordered(0, N, 1, N, 61, J2=0.3)
    env = envs(N)
    b = ed.Basis(env, mag)
    Jt = torch.tensor(J, dtype=torch.float64, requires_grad=True)
    Dt = torch.tensor(D, dtype=torch.float64, requires_grad=True)
    ht = torch.tensor(hi, dtype=torch.float64, requires_grad=True)
    E = ed.ground_state_energy(env, b, pairs, Jt, Dt, ht)
    E.backward()
    H = dense_model(N, mag, pairs, J, D, hi).dense()
    w, U = np.linalg.eigh(H)
    assert abs(E.item() - w[0]) <= 1e-10 * abs(w[0])
    M = dense_model(N, mag, pairs, J, D, hi)
    u = U[:, 0].astype(np.complex128)
    for q in (0, 3, 12):
        i, j = int(pairs[q][0]), int(pairs[q][1])
        xy = 0.5 * (M.expect(1, i, j, u) + M.expect(2, i, j, u)).real
        assert abs(Jt.grad[q].item() - xy) <= 1e-9
        assert abs(Dt.grad[q].item() - M.expect(0, i, j, u).real) <= 1e-9
    assert abs(J @ Jt.grad.numpy() + D @ Dt.grad.numpy() + hi @ ht.grad.numpy() - w[0]) <= 1e-9 * abs(w[0])


def test_c4_square_4x6_gradients(ed, envs):
    """4x6 J1-J2 (N=24, Sz=0, dim 2,704,156), per-bond couplings
    J_b = base_b (1 + 0.1 z_b), fields U[-0.5, 0.5]: dE0/dtheta and the
    gradient of the lowest-4 eigenvalue sum against central differences
    (step 1e-5) of the device energies, 1e-6 relative."""
    N, mag = 24, 0
    pairs, J, D, hi = disordered(1, N, 4, 6, 71, J2=0.5)
    env = envs(N)
    b = ed.Basis(env, mag)

    def solve(Jx, Dx, hx, nev=4):
        h = ed.Hamiltonian.from_bonds(env, b, pairs, Jx, Dx)
        h.build_diag(env)
        h.build_off_diag(env)
        h.build_disorder(env, hx)
        eps = ed.Solver.SolverInit(h, nev, 20)
        ed.Solver.EPSSetTolerances(eps, 1e-13)
        ed.Solver.solve(env, eps)
        return h, eps

    h, eps = solve(J, D, hi)
    e = [ed.Solver.eigenvalue(eps, n)[0] for n in range(4)]
    _, v0, _ = ed.Solver.solution(eps, 0)
    dJ, dD, dh = ed.Adjoint.energy_gradient(b, pairs, v0)
    sJ, sD, sh = ed.Adjoint.eigenvalue_sum_gradient(eps, pairs, 4)
    # sum rules: E = sum_b J_b <XY_b> + D_b <ZZ_b> + sum_i h_i <S^z_i>
    assert abs(J @ dJ + D @ dD + hi @ dh - e[0]) <= 1e-10 * abs(e[0])
    assert abs(J @ sJ + D @ sD + hi @ sh - sum(e)) <= 1e-10 * abs(sum(e))
    ed.Solver.SolverClean(eps)
    d = 1e-5

    def energies(Jx, Dx, hx):
        _, ep = solve(Jx, Dx, hx)
        out = [ed.Solver.eigenvalue(ep, n)[0] for n in range(4)]
        ed.Solver.SolverClean(ep)
        return np.array(out)

    for q in (0, 30):
        Jp, Jm = J.copy(), J.copy()
        Jp[q] += d
        Jm[q] -= d
        Ep, Em = energies(Jp, D, hi), energies(Jm, D, hi)
        fd0 = (Ep[0] - Em[0]) / (2 * d)
        fds = (Ep.sum() - Em.sum()) / (2 * d)
        assert abs(fd0 - dJ[q]) <= 1e-6 * max(1.0, abs(fd0)), (q, fd0, dJ[q])
        assert abs(fds - sJ[q]) <= 1e-6 * max(1.0, abs(fds)), (q, fds, sJ[q])
    hp, hm = hi.copy(), hi.copy()
    hp[5] += d
    hm[5] -= d
    fd0 = (energies(J, D, hp)[0] - energies(J, D, hm)[0]) / (2 * d)
    assert abs(fd0 - dh[5]) <= 1e-6 * max(1.0, abs(fd0))


def test_c4_square_4x4_minres_and_correlation_gradient(ed, envs):
    """4x4 J1-J2 (N=16, Sz=0, dim 12,870) with per-bond couplings
    J_b = base_b (1 + 0.1 z_b), D_b = J_b, fields U[-0.5, 0.5]: MINRES for
    (H - E0) lam = P (O - <O>) psi0, O = S_0 . S_far, reaches relres <= 1e-11,
    lam is orthogonal to psi0 and solves the projected system against the
    oracle's explicit matrix (1e-9 relative); d<O>/dtheta for two bonds (J and
    D) and one field against central differences (step 1e-4) of device
    expectation values, 1e-6 relative."""
    N, lx, ly, mag = 16, 4, 4, 0
    pairs, J, D, hi = disordered(1, N, lx, ly, 81, J2=0.5)
    env = envs(N)
    b = ed.Basis(env, mag)
    far = (lx // 2) * ly + ly // 2

    def solve(Jx, Dx, hx):
        h = ed.Hamiltonian.from_bonds(env, b, pairs, Jx, Dx)
        h.build_diag(env)
        h.build_off_diag(env)
        h.build_disorder(env, hx)
        eps = ed.Solver.SolverInit(h, 2, 20)
        ed.Solver.EPSSetTolerances(eps, 1e-13)
        ed.Solver.solve(env, eps)
        e0, v, _ = ed.Solver.solution(eps, 0)
        ed.Solver.SolverClean(eps)
        return h, e0, v

    def expval(Jx, Dx, hx):
        _, _, v = solve(Jx, Dx, hx)
        vn = v / np.sqrt(np.real(v.conj().dot(v).item()))
        return float(np.real(ed.SiSj(env, b).ExpectVal(env, 0, far, vn)))

    h, e0, v = solve(J, D, hi)
    obs = [(1.0, ed.Adjoint.SISJ, 0, far)]
    val, dJ, dD, dh, info = ed.Adjoint.expectation_gradient(h, pairs, e0, v, obs, tol=1e-12)
    assert info['relres'] <= 1e-11, info
    assert abs(val - expval(J, D, hi)) <= 1e-10
    # the adjoint solve itself, against the oracle's explicit matrix
    psi = v.cpu().numpy()
    psi = psi / np.linalg.norm(psi)
    opsi = ed.Adjoint.apply_observable(b, obs, psi).cpu().numpy()
    rhs = opsi - np.vdot(psi, opsi) * psi
    lam, its, rel = ed.Adjoint.minres(h, e0, rhs, q=psi, tol=1e-12)
    lam = lam.cpu().numpy()
    M = dense_model(N, mag, pairs, J, D, hi)
    assert abs(np.vdot(psi, lam)) <= 1e-10 * np.linalg.norm(lam)
    r = M.apply(lam) - e0 * lam - rhs
    r = r - np.vdot(psi, r) * psi
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(rhs), (np.linalg.norm(r), its, rel)
    d = 1e-4
    for q in (3, 40):
        Jp, Jm = J.copy(), J.copy()
        Jp[q] += d
        Jm[q] -= d
        fd = (expval(Jp, D, hi) - expval(Jm, D, hi)) / (2 * d)
        assert abs(fd - dJ[q]) <= 1e-6 * max(1.0, abs(fd)), (q, fd, dJ[q])
        Dp, Dm = D.copy(), D.copy()
        Dp[q] += d
        Dm[q] -= d
        fd = (expval(J, Dp, hi) - expval(J, Dm, hi)) / (2 * d)
        assert abs(fd - dD[q]) <= 1e-6 * max(1.0, abs(fd)), (q, fd, dD[q])
    hp, hm = hi.copy(), hi.copy()
    hp[5] += d
    hm[5] -= d
    fd = (expval(J, D, hp) - expval(J, D, hm)) / (2 * d)
    assert abs(fd - dh[5]) <= 1e-6 * max(1.0, abs(fd)), (fd, dh[5])
