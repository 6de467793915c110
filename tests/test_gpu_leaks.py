"""Device-memory leak check, the counterpart of the reference tests'
``-malloc_dump`` (tests/unit_tests/meson.build:26): a full cycle of the
public API (context, bases, Hamiltonian in every H.v mode, both solver
storage forms, correlations, DSF, the batched sweep, the adjoint solver)
returns every byte it allocated.  The first cycle is a warm-up: the H.v
kernels compiled at run time are loaded once per operator structure and kept
for the process, and torch's caching allocator keeps its blocks until
empty_cache()."""
import gc

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def ed():
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300
    return lsquantumed_gb300


def _work(ed):
    import torch
    env = ed.Environment(nspins=16)
    lat = ed.square2D(env, 4, 4)
    b0 = ed.Basis(env, 0)
    b1 = ed.Basis(env, 1)
    h = ed.Hamiltonian(env, b0, lat, 1.0, 1.0, 0.5, 0.5)
    h.build_diag(env)
    h.build_off_diag(env)
    x = oracle.start_vector(2, b0.size)
    for acc in ('exact', 'fp64', 'fixed64'):
        h.set_accumulation(acc)
        h.apply(x)
    for v in ('u4-b6', 'jit', 'jit-b3', 'auto'):
        h.set_hv_variant(v)
        h.apply(x)
        h.apply_real(x.real.copy())
    h.apply_host(x)
    h.build_csr()
    h.set_mode('csr')
    h.apply(x)
    h.set_mode('matrix_free')
    # real-storage solve (seeded start) and complex path (complex start)
    eps = ed.Solver.SolverInit(h, 3, 16)
    ed.Solver.EPSSetTolerances(eps, 1e-10)
    eps.set_restart_arithmetic('pair')
    ed.Solver.solve(env, eps)
    e0, psi, _ = ed.Solver.solution(eps, 0)
    ed.Solver.solution_host(eps, 1)
    ed.Solver.SolverClean(eps)
    eps = ed.Solver.SolverInit(h, 2, 16)
    eps.set_initial_vector(x)
    ed.Solver.solve(env, eps)
    ed.Solver.SolverClean(eps)
    ed.SiSj(env, b0).AllPairs(psi)
    # DSF coefficients for Sqz (same sector) and Sqp (sector 0 -> 1)
    h1 = ed.Hamiltonian(env, b1, lat, 1.0, 1.0, 0.5, 0.5)
    h1.build_diag(env)
    h1.build_off_diag(env)
    eps1 = ed.Solver.SolverInit(h1, 2, 16)
    ed.Solver.solve(env, eps1)
    vecs = torch.stack([ed.Solver.solution(eps1, n)[1] for n in range(2)])
    c = ed.Phys.dsf_coefficients(env, b0, b1, 1, psi, vecs)
    ed.Solver.SolverClean(eps1)
    pos = ed.Phys.site_positions(lat)
    ed.Phys.dsf_spectrum(env, c, np.array([0.5, 0.7]), pos, ed.Phys.q_grid(lat)[:3], nw=101)
    # batched sweep
    bt = ed.DisorderBatch(h, np.stack([oracle.rd_hi(s, 16, -1.0, 1.0) for s in range(3)]))
    bt.solve(nev=1, ncv=12, tol=1e-9)
    bt.eigenvector(1, 0)
    del bt
    # adjoint: energy gradient and one shifted solve
    pairs = np.asarray(lat.nn_pairs, dtype=np.int32)
    ed.Adjoint.energy_gradient(b0, pairs, psi)
    rhs = ed.Adjoint.apply_observable(b0, [(1.0, ed.capi.ED_TERM_SISJ, 0, 1)], psi)
    ed.Adjoint.minres(h, e0, rhs, q=psi, tol=1e-10)
    env.synchronize()


def _cycle(ed):
    """One cycle; every handle is released by reference counting when _work
    returns (objects keep their Environment alive, so the context goes last)."""
    import torch
    _work(ed)
    gc.collect()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def test_no_device_memory_growth(ed):
    import torch
    _cycle(ed)
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        _cycle(ed)
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 <= 4 << 20, (free0, free1)
