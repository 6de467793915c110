#!/usr/bin/env python3
"""Benchmark: N=30 (6x5 square, J1=1, J2=0.55, Delta=1, Sz=0) Krylov-Schur
eigensolve, lowest 4 eigenpairs, ncv=16, eps_tol=1e-9, matrix-free H.v.

One step = one full eigensolve (start vector to converged eigenpairs) with the
Hamiltonian resident in HBM.  Prints one JSON line (see the keys below).

  python bench.py [--steps K] [--warmup W] [--impl ours|reference] [--workload c5|c2|c1]

--impl reference times the CPU restatement of the reference path (the oracle
port; the PETSc/SLEPc reference cannot be built here) on the host cores.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'eigensolve s & H·v GB/s at N=30; disorder samples/s batched vs plain @res1e-9'

WORKLOADS = {
    # name: (lattice, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol)
    'c5': ('square2D', 30, 6, 5, 1.0, 1.0, 0.55, 0.55, 0, 4, 16, 1e-9),
    'c2': ('square2D', 20, 4, 5, 1.0, 1.0, 0.5, 0.5, 0, 10, 0, 1e-9),
    'c1': ('chain1D', 16, 1, 16, 1.0, 1.0, 0.0, 0.0, 0, 1, 0, 1e-9),
    # same family, sized for profiler captures (vectors 0.64 GB, above L2)
    'p28': ('square2D', 28, 4, 7, 1.0, 1.0, 0.55, 0.55, 0, 4, 16, 1e-9),
}
# H.v applications the Krylov-Schur run needs on each workload (seed 0), as
# measured by the device run; the CPU restatement runs the same algorithm from
# the same start vector, so its count is the same.  Used only to extrapolate
# the bounded CPU sample of the reference arm (a workload not listed uses 300).
NHV = {'c5': 334}


def _rank_info():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rk = int(os.environ.get('RANK', '0'))
    lr = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rk, lr


def shard_units(n, rank, world):
    """Round-robin partition of n independent units (disorder seeds) over the
    ranks: each rank solves its own seeds, no data-path collective."""
    return list(range(rank, n, world))


def dist_reduce(value, ws, op='max'):
    """MAX or SUM of a host scalar over the ranks (gloo; identity when ws == 1)."""
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == 'max' else dist.ReduceOp.SUM)
    return float(t[0])


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def kbar(N, nup, pairs):
    """Mean off-diagonal entries per row: sum over distinct bonds of
    P(bond antiparallel) = 2 C(N-2, nup-1) / C(N, nup)."""
    masks = {(min(i, j), max(i, j)) for i, j in pairs if i != j}
    p = 2 * math.comb(N - 2, nup - 1) / math.comb(N, nup)
    return len(masks) * p


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix='.csv')
            os.close(fd)
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.device), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': []}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(',')]
            if len(f) < 8:
                continue
            try:
                rows.append((float(f[0]), float(f[1]), f[4], f[5], f[6], f[7]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return out
        sm = sorted(r[0] for r in rows)
        out['sm_mhz'] = sm[len(sm) // 2]
        out['sm_max_mhz'] = max(r[1] for r in rows)
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for k, nm in enumerate(names):
            if any(r[2 + k].lower().startswith('active') for r in rows):
                out['reasons'].append(nm)
        out['samples'] = len(rows)
        return out


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port on the host cores, bounded sample.
# ---------------------------------------------------------------------------
class CpuSample:
    """CSR SpMV (int64 columns, complex128 values, the reference's matrix
    layout) and one CGS pass over 12 vectors on all host threads, at the
    largest size of the same family whose explicit matrix fits host memory
    (N=24 4x6 for the N=30 workload).  Per-row costs are scaled to the
    workload's basis and multiplied by the solver's H.v count.  The matrix
    build is setup, not timed (as the device run excludes its own setup)."""

    def __init__(self, wl):
        import numpy as np
        import oracle
        self.wl = wl
        ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
        self.N, self.mag = N, mag
        self.sN, self.slx, self.sly = (24, 4, 6) if N > 24 else (N, lx, ly)
        self.lt = oracle.SQUARE2D if ltype == 'square2D' else oracle.CHAIN1D
        self.M = oracle.Model(self.lt, self.sN, self.slx, self.sly, 0, J1, D1, J2, D2)
        self.nnz = self.M.build(3)
        n = self.M.dim
        self.x = oracle.start_vector(1, n)
        # an orthonormal basis, so repeated CGS passes on w stay bounded
        q, _ = np.linalg.qr(np.stack([oracle.start_vector(10 + i, n) for i in range(12)]).T)
        self.V = np.ascontiguousarray(q.T)
        self.w = oracle.start_vector(2, n)
        nn, nnn = oracle.bond_pairs(self.lt, N, lx, ly)
        self.nnz_row_f = 1 + kbar(N, mag + N // 2, list(map(tuple, nn)) + (list(map(tuple, nnn)) if J2 else []))
        self.M.apply(self.x)  # warm

    def run(self, nhv, budget_s=8.0):
        import oracle
        n = self.M.dim
        t0 = time.perf_counter()
        reps = 0
        while True:
            self.M.apply(self.x)
            reps += 1
            if time.perf_counter() - t0 > budget_s / 2 or reps >= 50:
                break
        t_spmv = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        creps = 0
        while True:
            oracle.cgs_step(self.V, self.w)
            creps += 1
            if time.perf_counter() - t0 > budget_s / 4 or creps >= 20:
                break
        t_cgs = (time.perf_counter() - t0) / creps
        full_dim = math.comb(self.N, self.mag + self.N // 2)
        nnz_row_s = self.nnz / n
        t_hv_full = t_spmv * (full_dim / n) * (self.nnz_row_f / nnz_row_s)
        # CGS with one refinement: two passes per step over ~12 vectors on average
        t_step = t_hv_full + 2 * t_cgs * (full_dim / n)
        return {
            'value': t_step * nhv, 'unit': 's', 'cores': oracle.get_threads(), 'kind': 'port',
            'sample': ('N=%d %dx%d explicit-CSR SpMV (%d reps, %.4f s each) + CGS pass over 12 vectors '
                       '(%.4f s), scaled to N=%d rows (x%.2f) and nnz/row (x%.3f), times %d H.v per solve'
                       % (self.sN, self.slx, self.sly, reps, t_spmv, t_cgs, self.N, full_dim / n,
                          self.nnz_row_f / nnz_row_s, nhv)),
        }


def run_reference(args):
    ws, rk, lr = _rank_info()
    if rk != 0:
        return 0
    wl = args.workload
    import oracle
    ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    nhv = NHV.get(wl)
    times = []
    res = None
    sample = CpuSample(wl) if N > 24 else None
    for step in range(args.warmup + args.steps):
        if sample is not None:
            res = sample.run(nhv or 300)
        else:
            t0 = time.perf_counter()
            lt = oracle.SQUARE2D if ltype == 'square2D' else oracle.CHAIN1D
            M = oracle.Model(lt, N, lx, ly, mag, J1, D1, J2, D2)
            M.build(3)
            r = M.eps_solve(nev=nev, ncv=ncv, tol=tol, seed=0, vectors=False)
            res = {'value': time.perf_counter() - t0, 'unit': 's', 'cores': oracle.get_threads(), 'kind': 'port',
                   'sample': 'full CPU eigensolve (CSR build + Krylov-Schur), nhv=%d' % r['nhv']}
        if step >= args.warmup:
            times.append(res['value'])
    v = sum(times) / len(times)
    res['value'] = v
    line = {'metric': METRIC, 'value': v, 'unit': 's', 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': v * 1e3, 'higher_is_better': False, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'c128', 'data': 'synthetic',
            'config': workload_config(wl), 'impl': 'reference', 'cpu_baseline': res,
            'e2e': {'value': v, 'unit': 's', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line))
    return 0


def workload_config(wl):
    ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    return {'workload': '%s %s N=%d (%dx%d) J1=%g J2=%g Delta=1 Sz=%d: lowest %d eigenpairs, ncv=%s, eps_tol=%g, '
                        'matrix-free complex128 H.v' % (wl, ltype, N, lx, ly, J1, J2, mag, nev, ncv or 'decide', tol),
            'nspins': N, 'lattice': ltype, 'lx': lx, 'ly': ly, 'J1': J1, 'J2': J2, 'Delta': 1.0, 'sz': mag,
            'nev': nev, 'ncv': ncv, 'eps_tol': tol, 'dim': math.comb(N, mag + N // 2), 'seed': 0,
            'l2': ('inputs larger than L2 (each vector %.2f GB)' if 16 * math.comb(N, mag + N // 2) > 129e6 else
                   'inputs smaller than L2, not flushed (each vector %.4f GB): an outputs/parity case, not the '
                   'headline workload') % (16 * math.comb(N, mag + N // 2) / 1e9)}


def workload_outputs(ed, env, b, lat, wl, eps, evals):
    """The measurements the C1 / C2 configurations ask for, from the last
    solve (outside the timed region).
    C1 (chain N=16): E0, <S_0.S_r> for every r, m^2_AF.
    C2 (4x5 J1-J2): all N^2 <S_i.S_j> and the DSF weights
    |<n|S^z_q|0>|^2 over the nev levels at q = (pi, pi) and (pi, 0), with
    r_i = (i // ly, i % ly); ly = 5 is odd, so q_y = pi is off the lattice's
    grid and the nearest grid value 4 pi / 5 is used (stated in the line)."""
    import numpy as np
    import torch
    N = env.nspins
    _, psi0, _ = ed.Solver.solution(eps, 0)
    out = {'E': [float(e) for e in evals]}
    t0 = time.perf_counter()
    if wl == 'c1':
        r = ed.SiSj(env, b).ExpectValPairs([(0, j) for j in range(N)], psi0)
        out['S0_Sr'] = [float(np.real(v)) for v in r]
        out['m2_af'] = float(np.real(ed.Phys.SquaredSubLattMagAF(env, b, ed.AF(lat), psi0)))
    else:
        C = ed.SiSj(env, b).AllPairs(psi0)
        out['sisj_sum'] = float(np.real(C.sum()))
        out['S0_S1'] = float(np.real(C[0, 1]))
        n = len(evals)
        V = torch.stack([ed.Solver.solution(eps, i)[1] for i in range(n)])
        c = ed.Phys.dsf_coefficients(env, b, b, 0, psi0, V)
        pos = ed.Phys.site_positions(lat)
        lx, ly = lat.nspins_x, lat.nspins_y
        q_grid = [(np.pi, 2 * np.pi * round(ly / 2 - 0.5) / ly), (np.pi, 0.0)]
        out['dsf'] = {'q_requested': [[np.pi, np.pi], [np.pi, 0.0]], 'q_used': [list(q) for q in q_grid],
                      'dE': [float(e - evals[0]) for e in evals],
                      'weights': [[float(w) for w in ed.Phys.dsf_weights(c, pos, q)] for q in q_grid]}
    torch.cuda.synchronize()
    out['seconds'] = time.perf_counter() - t0
    return out


def c3_cpu_sample(fields, sectors, N, J1, J2, nev, tol):
    """The oracle's CPU eigensolve (explicit CSR in the reference layout,
    Krylov-Schur, all host threads) of the chain with each field realisation
    in each sector, as one disorder-sweep sample each: (samples/s, threads,
    {sector: [lowest nev eigenvalues per realisation]})."""
    import oracle
    t0 = time.perf_counter()
    evals = {}
    for mag in sectors:
        evals[mag] = []
        for hi in fields:
            M = oracle.Model(oracle.CHAIN1D, N, 1, N, mag, J1, 1.0, J2, J2)
            M.build(3, hi)
            r = M.eps_solve(nev=nev, ncv=16, tol=tol, seed=0, vectors=False)
            evals[mag].append(r['evals'][:nev])
    dt = time.perf_counter() - t0
    return len(sectors) * len(fields) / dt, oracle.get_threads(), evals


def run_disorder(args):
    """C3: disorder sweep, chain N=20 (J1=1, J2=0.2, Delta=1), h_i ~ U[-2, 2]
    from mt19937_64(seed) for seed = 0..511 (RandomDisorder::hi_init with
    srand_seq[k] = seed), Sz = 0, 1, 2: 1536 solves (lowest 2 pairs,
    eps_tol 1e-9).  Batched: one lockstep batch per sector.  Plain: the same
    solves issued one at a time (a bounded subset, timed per solve)."""
    import numpy as np
    import torch
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300 as ed
    N, J1, J2, W, nev, tol = 20, 1.0, 0.2, 2.0, 2, 1e-9
    ws, rk, lr = _rank_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group('gloo')
    torch.cuda.set_device(lr)
    nseeds = args.seeds
    mine = shard_units(nseeds, rk, ws)  # this rank's seeds (weak scaling: every rank a share)
    env = ed.Environment(nspins=N, device=lr)
    fields = np.stack([ed.random_fields(sd, N, -W, W) for sd in mine])
    sectors = (0, 1, 2)
    hams = {}
    for mag in sectors:
        b = ed.Basis(env, mag)
        h = ed.Hamiltonian(env, b, ed.chain1D(env), J1, 1.0, J2, J2)
        h.build_diag(env)
        h.build_off_diag(env)
        hams[mag] = (b, h)
    # batched
    for _ in range(1 if args.warmup else 0):  # warm-up on a small batch
        bt = ed.DisorderBatch(hams[0][1], fields[:8])
        bt.solve(nev=nev, ncv=16, tol=tol, seed=0)
        del bt
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    k0 = env.kernel_count()
    t0 = time.perf_counter()
    max_err, its, bad = 0.0, [], 0
    batch_evals = {}
    for mag in sectors:
        bt = ed.DisorderBatch(hams[mag][1], fields)
        bt.set_restart_arithmetic(args.restart)
        r = bt.solve(nev=nev, ncv=16, tol=tol, seed=0)
        max_err = max(max_err, float(r['errs'].max()))
        bad += int((r['nconv'] < nev).sum())
        its.append(r['its'])
        batch_evals[mag] = r['evals']
        del bt
    torch.cuda.synchronize()
    t_batch = dist_reduce(time.perf_counter() - t0, ws, 'max')
    launches = env.kernel_count() - k0
    max_err = dist_reduce(max_err, ws, 'max')
    bad = int(dist_reduce(bad, ws, 'sum'))
    nsolve = nseeds * len(sectors)
    if rk != 0:
        return 0
    # plain: one solve at a time on a subset
    nplain = min(args.plain_sample, len(mine))
    t0 = time.perf_counter()
    agree = True
    for mag in sectors:
        b, _ = hams[mag]
        for sd in range(nplain):
            h = ed.Hamiltonian(env, b, ed.chain1D(env), J1, 1.0, J2, J2)
            h.build_diag(env)
            h.build_off_diag(env)
            h.build_disorder(env, fields[sd])
            eps = ed.Solver.SolverInit(h, nev, 16)
            ed.Solver.EPSSetTolerances(eps, tol)
            ed.Solver.solve(env, eps)
            for i in range(nev):
                e, _ = ed.Solver.eigenvalue(eps, i)
                agree &= abs(e - batch_evals[mag][sd][i]) <= 1e-8 * abs(e)
            ed.Solver.SolverClean(eps)
    torch.cuda.synchronize()
    t_plain = (time.perf_counter() - t0) / (nplain * len(sectors))
    # CPU baseline: the oracle port on a bounded subset of the same solves
    cpu = None
    if not args.no_cpu:
        try:
            k = max(1, min(args.cpu_seeds, len(mine)))
            sps, cores, cev = c3_cpu_sample(fields[:k], sectors, N, J1, J2, nev, tol)
            cagree = all(abs(cev[mag][i][q] - batch_evals[mag][i][q]) <= 1e-8 * abs(cev[mag][i][q])
                         for mag in sectors for i in range(k) for q in range(nev))
            cpu = {'value': sps, 'unit': 'samples/s', 'cores': cores, 'kind': 'port',
                   'sample': '%d seeds x %d sectors: full CPU eigensolves (explicit CSR build + Krylov-Schur, '
                             'nev=2, tol 1e-9), the rate extrapolated to the sweep' % (k, len(sectors)),
                   'eigenvalues_agree_1e-8': bool(cagree)}
        except Exception as ex:  # reported, never fatal
            cpu = {'value': None, 'unit': 'samples/s', 'cores': None, 'kind': 'port', 'sample': 'failed: %s' % ex}
    line = {'metric': METRIC, 'workload': 'c3', 'value': nsolve / t_batch, 'unit': 'samples/s',
            'higher_is_better': True, 'n_gpus': ws, 'steps': 1, 'warmup': args.warmup,
            'scaling': 'strong',  # the 1,536 solves are split over the ranks by seed
            'batched': {'samples_per_s': nsolve / t_batch, 'seconds': t_batch, 'solves': nsolve,
                        'restarts_per_sector': its, 'max_rel_residual': max_err, 'unconverged': bad,
                        'gpu_launches': launches, 'restart_arithmetic': args.restart},
            'plain': {'samples_per_s': 1.0 / t_plain, 'seconds_per_solve': t_plain,
                      'sample': '%d seeds x %d sectors, one solve at a time' % (nplain, len(sectors))},
            'batched_over_plain': (nsolve / t_batch) * t_plain,
            'cpu_baseline': cpu,
            'eigenvalues_agree_1e-8': bool(agree), 'dtype': 'f64', 'data': 'synthetic',
            'dtype_note': 'FP64 real storage of the Krylov basis (the complex128 solve of the reference with its '
                          'exactly-zero imaginary parts dropped); H.v sums in exact int64 fixed point; restart '
                          'products as float pairs on the FP32 units from 2^22 states up',
            'config': {'workload': 'c3 chain1D N=20 J1=1 J2=0.2 Delta=1, h_i~U[-2,2] seeds 0..%d, Sz=0,1,2, '
                                   'nev=2, ncv=16, eps_tol=1e-9' % (nseeds - 1), 'dims': [b.size for b, _ in hams.values()]}}
    print(json.dumps(line))
    return 0


def hv_bytes_per_row(kb, mode):
    """Algorithmic bytes per row of one matrix-free H.v: x_s + the gathered
    x_s' (k-bar entries) + y_s + state (4) + diagonal (8).
    mode 'complex': complex128 vectors, 16-byte gathers;
    'real_gathers': complex128 vectors whose imaginary parts are zero, the
    fixed-point copy holds real parts (8-byte gathers);
    'real_storage': vectors stored as their real parts (the real-mode solve):
    8-byte x_s, gathers and y_s."""
    vec, gat = {'complex': (16, 16), 'real_gathers': (16, 8), 'real_storage': (8, 8)}[mode]
    return vec + gat * kb + vec + 4 + 8


def run_hv_only(args):
    """Time the matrix-free H.v alone (K launches after W warm-up launches,
    CUDA events on the launching stream) for the workload's Hamiltonian."""
    import numpy as np
    import torch
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300 as ed
    wl = args.workload
    ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    env = ed.Environment(nspins=N)
    b = ed.Basis(env, mag)
    lat = ed.square2D(env, lx, ly) if ltype == 'square2D' else ed.chain1D(env)
    H = ed.Hamiltonian(env, b, lat, J1, D1, J2, D2)
    H.build_diag(env)
    H.build_off_diag(env)
    H.set_accumulation(args.acc)
    if args.variant != 'auto':
        H.set_hv_variant(args.variant)
    dim = b.size
    if args.real_storage:
        x = torch.empty(dim, dtype=torch.float64, device='cuda').uniform_(-1, 1)
        apply = H.apply_real
    else:
        x = torch.empty(dim, dtype=torch.complex128, device='cuda')
        x.real.uniform_(-1, 1)
        if args.real_input:
            x.imag.zero_()
        else:
            x.imag.uniform_(-1, 1)
        apply = H.apply
    x /= torch.linalg.vector_norm(x)
    y = torch.empty_like(x)
    for _ in range(args.warmup):
        apply(x, out=y)
    torch.cuda.synchronize()
    env.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream()
    e0.record(stream)
    for _ in range(args.steps):
        apply(x, out=y)
    e1.record(stream)
    torch.cuda.synchronize()
    n_hv, ms_hv = env.profile_read()
    env.profile(False)
    pairs = list(map(tuple, lat.nn_pairs)) + (list(map(tuple, lat.nnn_pairs)) if J2 else [])
    real_mode = (args.real_input or args.real_storage) and args.acc == 'fixed64'
    mode = 'real_storage' if args.real_storage else ('real_gathers' if real_mode else 'complex')
    bytes_row = hv_bytes_per_row(kbar(N, b.nspins_up, pairs), mode)
    ms = ms_hv / max(n_hv, 1)
    peak, _ = measured_peaks()
    gbs = dim * bytes_row / (ms * 1e-3) / 1e9
    print(json.dumps({'mode': 'hv-only', 'workload': wl, 'acc': args.acc, 'real_input': bool(args.real_input),
                      'real_storage': bool(args.real_storage),
                      'dim': dim, 'launches': n_hv, 'ms_per_hv': ms,
                      'ms_per_step_events': e0.elapsed_time(e1) / args.steps, 'algorithmic_gbs': gbs,
                      'frac_of_measured_hbm': gbs / peak, 'bytes_per_row': bytes_row,
                      'variant': H.hv_variant(False)}))
    return 0


def run_ours(args):
    import numpy as np
    import torch
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300 as ed

    ws, rk, lr = _rank_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group('gloo')
    torch.cuda.set_device(lr)
    wl = args.workload
    ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    env = ed.Environment(nspins=N, device=lr)
    b = ed.Basis(env, mag)
    lat = ed.square2D(env, lx, ly) if ltype == 'square2D' else ed.chain1D(env)
    H = ed.Hamiltonian(env, b, lat, J1, D1, J2, D2)
    H.build_diag(env)
    H.build_off_diag(env)
    dim = b.size

    def one_solve():
        eps = ed.Solver.SolverInit(H, nev, ncv if ncv else ed.PETSC_DEFAULT)
        ed.Solver.EPSSetTolerances(eps, tol, 0)
        eps.set_restart_arithmetic(args.restart)
        nconv = ed.Solver.solve(env, eps)
        return eps, nconv

    for _ in range(args.warmup):
        eps, _ = one_solve()
        ed.Solver.SolverClean(eps)
    stream = torch.cuda.current_stream()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(lr)
    sampler.start()
    k0 = env.kernel_count()
    env.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    last = None
    for _ in range(args.steps):
        if last is not None:
            ed.Solver.SolverClean(last[0])
        last = one_solve()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    n_hv, ms_hv = env.profile_read()
    env.profile(False)
    launches = env.kernel_count() - k0
    eps, nconv = last
    st = eps.stats()
    evals, errs = [], []
    for i in range(min(nev, st['nreported'])):
        e, err = ed.Solver.eigenvalue(eps, i)
        evals.append(e)
        errs.append(err)
    # all N^2 <S_i.S_j> in the ground state (measured after the timed solves)
    sisj = None
    if not args.no_sisj:
        _, psi0, _ = ed.Solver.solution(eps, 0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        C = ed.SiSj(env, b).AllPairs(psi0)
        torch.cuda.synchronize()
        sisj = {'seconds': time.perf_counter() - t0, 'pairs': N * N,
                'sum_check': float(np.real(C.sum())),  # <S_tot^2> = S(S+1) = 0 for a singlet ground state
                'S0_S1': float(np.real(C[0, 1]))}
        del psi0
    outputs = workload_outputs(ed, env, b, lat, wl, eps, evals) if wl in ('c1', 'c2') else None
    ed.Solver.SolverClean(eps)
    ms_step = dist_reduce(ms / args.steps, ws, 'max')

    # roofline of the dominant kernel (H.v): algorithmic bytes per launch
    pairs = list(map(tuple, lat.nn_pairs)) + (list(map(tuple, lat.nnn_pairs)) if J2 else [])
    kb = kbar(N, b.nspins_up, pairs)
    # the solve starts from a real vector (H real symmetric): the basis is
    # stored as its real parts and every H.v reads and writes 8-byte entries
    bytes_row = hv_bytes_per_row(kb, 'real_storage')
    bytes_row_complex = hv_bytes_per_row(kb, 'complex')
    hv_ms = ms_hv / max(n_hv, 1)
    achieved = dim * bytes_row / (hv_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic, traffic_note = None, None
    tp = os.path.join(ROOT, 'profiles', 'hv_traffic.json')
    if os.path.exists(tp):
        try:
            tj = json.load(open(tp)).get(wl)
            if tj:
                traffic = tj.get('dram_bytes_per_launch')
                traffic_note = tj.get('note')
        except Exception:
            traffic = None

    # e2e through the public API with host buffers (pinned), one step: basis,
    # Hamiltonian, start vector uploaded from host memory, solve, eigenvectors
    # read back into host memory.
    e2e = None
    if not args.no_e2e:
        start_host = torch.empty(dim, dtype=torch.complex128, pin_memory=True)
        start_host.numpy()[:] = start_vector_host(dim)
        out_host = [torch.empty(dim, dtype=torch.complex128, pin_memory=True) for _ in range(nev)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b2 = ed.Basis(env, mag)
        lat2 = ed.square2D(env, lx, ly) if ltype == 'square2D' else ed.chain1D(env)
        H2 = ed.Hamiltonian(env, b2, lat2, J1, D1, J2, D2)
        H2.build_diag(env)
        H2.build_off_diag(env)
        eps2 = ed.Solver.SolverInit(H2, nev, ncv if ncv else ed.PETSC_DEFAULT)
        ed.Solver.EPSSetTolerances(eps2, tol, 0)
        eps2.set_restart_arithmetic(args.restart)
        eps2.set_initial_vector(start_host)
        ed.Solver.solve(env, eps2)
        vals2 = []
        for i in range(nev):
            e, err = ed.Solver.eigenvalue(eps2, i)
            vals2.append(e)
            ed.Solver.solution_host(eps2, i, out=out_host[i])
        torch.cuda.synchronize()
        t_e2e = time.perf_counter() - t0
        ed.Solver.SolverClean(eps2)
        del H2, b2
        e2e = {'value': t_e2e, 'unit': 's', 'h2d_bytes_per_step': int(16 * dim + 8 * 2 * len(pairs)),
               'd2h_bytes_per_step': int(16 * dim * nev), 'steps': 1,
               'eigenvalues_match_device_run': bool(np.allclose(vals2, evals, rtol=1e-10, atol=0))}

    cpu = None
    if rk == 0 and not args.no_cpu:
        try:
            cpu = CpuSample(wl).run(st['nhv']) if N > 24 else None
            if cpu is None:
                import oracle
                lt = oracle.SQUARE2D if ltype == 'square2D' else oracle.CHAIN1D
                t0 = time.perf_counter()
                M = oracle.Model(lt, N, lx, ly, mag, J1, D1, J2, D2)
                M.build(3)
                r = M.eps_solve(nev=nev, ncv=ncv, tol=tol, seed=0, vectors=False)
                cpu = {'value': time.perf_counter() - t0, 'unit': 's', 'cores': oracle.get_threads(),
                       'kind': 'port', 'sample': 'full CPU eigensolve, nhv=%d' % r['nhv']}
        except Exception as ex:  # reported, never fatal
            cpu = {'value': None, 'unit': 's', 'cores': None, 'kind': 'port', 'sample': 'failed: %s' % ex}

    if rk != 0:
        return 0
    line = {
        'metric': METRIC, 'value': ms_step / 1e3, 'unit': 's', 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_step, 'higher_is_better': False, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': workload_config(wl),
        'dtype_note': 'FP64 real storage of the Krylov basis (the complex128 solve of the reference with its '
                  'exactly-zero imaginary parts dropped); H.v sums in exact int64 fixed point; restart '
                  'products as float pairs on the FP32 units from 2^22 states up',
        'e2e': e2e, 'gpu_launches': launches,
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                     'traffic': traffic,
                     'kernel': 'matrix-free H.v in real storage: two-table-rank kernel (k_hv_jit*_r when '
                               'hv_variant is jit*, else k_hv_lin); its fixed-point input comes from the '
                               'preceding scaling pass (k_scale_quantize_r), else k_max_exponent_r + '
                               'k_quantize64_r inside the timed launch',
                     'hv_variant': {'plain': H.hv_variant(False), 'fused_dot': H.hv_variant(True)},
                     'traffic_note': traffic_note, 'peak_kind': peak_kind,
                     'bytes_per_row': bytes_row, 'bytes_per_row_complex_input': bytes_row_complex,
                     'rows_per_launch': dim, 'avg_launch_ms': hv_ms,
                     'launches_timed': n_hv},
        'hv_gbs': achieved, 'sisj_all_pairs': sisj, 'outputs': outputs,
        'solver': {'nconv': nconv, 'its': st['its'], 'nhv': st['nhv'] // 1, 'ortho_passes': st['ortho_passes'],
                   'restart_arithmetic': args.restart,
                   'eigenvalues': evals,
                   'rel_residuals': errs},
        'clocks': clocks, 'cpu_baseline': cpu,
    }
    print(json.dumps(line))
    return 0


def start_vector_host(n, seed=0):
    """The solver's seeded start vector, generated on the host for the
    end-to-end run: re ~ U[-1,1) from splitmix64, imaginary parts zero (the
    solver starts from a real vector)."""
    import numpy as np
    i = np.arange(n, dtype=np.uint64)
    base = np.uint64((seed * 0xD1B54A32D192ED03) & 0xFFFFFFFFFFFFFFFF)

    def sm(z):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))
    with np.errstate(over='ignore'):
        h1 = sm(base + np.uint64(2) * i)
    u1 = (h1 >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (2.0 * u1 - 1.0).astype(np.complex128)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=2)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default='c5', choices=sorted(WORKLOADS) + ['c3'])
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-sisj', action='store_true', help='skip the all-pairs <S_i.S_j> measurement')
    ap.add_argument('--real-input', action='store_true', help='--hv-only with a real input vector')
    ap.add_argument('--restart', default='auto', choices=('auto', 'fp64', 'pair'),
                    help='restart-combination products of the real-storage solve (auto: float pairs from 2^22 states)')
    ap.add_argument('--real-storage', action='store_true',
                    help='--hv-only on real vectors in real storage (float64, as inside the solve)')
    ap.add_argument('--variant', default='auto', help='--hv-only: force an H.v launch variant (default: autotuner)')
    ap.add_argument('--hv-only', action='store_true', help='time the H.v kernel alone')
    ap.add_argument('--seeds', type=int, default=512, help='disorder seeds (c3)')
    ap.add_argument('--cpu-seeds', type=int, default=4, help='seeds of the C3 CPU baseline sample (x 3 sectors)')
    ap.add_argument('--plain-sample', type=int, default=16, help='seeds per sector solved one at a time (c3)')
    ap.add_argument('--acc', default='exact', choices=['exact', 'fixed64', 'fp64'], help='H.v accumulation')
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == 'reference':
        return run_reference(args)
    if args.hv_only:
        return run_hv_only(args)
    if args.workload == 'c3':
        return run_disorder(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
