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
DTYPE_NOTE = ('FP64 real storage of the Krylov basis (the complex128 solve of the reference with its exactly-zero '
              'imaginary parts dropped); H.v sums in exact int64 fixed point (error below 2^-57 of max|x| per '
              'entry); Gram-Schmidt and restart products FP64 or exact (every product FP64 or better)')

WORKLOADS = {
    # name: (lattice, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol)
    'c5': ('square2D', 30, 6, 5, 1.0, 1.0, 0.55, 0.55, 0, 4, 16, 1e-9),
    'c2': ('square2D', 20, 4, 5, 1.0, 1.0, 0.5, 0.5, 0, 10, 0, 1e-9),
    'c1': ('chain1D', 16, 1, 16, 1.0, 1.0, 0.0, 0.0, 0, 1, 0, 1e-9),
    # same family, sized for profiler captures (vectors 0.64 GB, above L2)
    'p28': ('square2D', 28, 4, 7, 1.0, 1.0, 0.55, 0.55, 0, 4, 16, 1e-9),
}


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
# CPU baseline: the oracle port on the host cores.
# ---------------------------------------------------------------------------
# The reference's CPU path assembles the explicit matrix (PETSc AIJ, 64-bit
# indices, complex128 values).  At N=30 that is about 235 GB, beyond host
# memory, so the measured CPU solve is the largest member of the same family
# that the bench can build and solve within its budget: the 4x6 J1-J2 lattice
# (N=24, 2.7M states, 138M stored entries, 3.3 GB).
CPU_SAMPLE = {'c5': (24, 4, 6), 'p28': (24, 4, 6)}
# H.v applications of the device solve of each workload from the seeded start
# vector; the reference arm runs in a process of its own with no device solve
# beside it, so it takes the count from here.  The GPU arm uses the count of
# its own solve instead.
NHV_DEVICE = {'c5': 334}


def host_info():
    """CPU model, logical cores, host RAM and the explicit-matrix sizes the
    reference would need (PETSc AIJ: 8-byte column + 16-byte value per entry,
    8 bytes per row pointer)."""
    model = None
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(':')
            if k.strip() in ('Model name', 'Vendor ID') and v.strip() and v.strip() != '-':
                model = (model + ' / ' if model else '') + v.strip()
    except Exception:
        pass
    ram = None
    try:
        for line in open('/proc/meminfo'):
            if line.startswith('MemTotal:'):
                ram = int(line.split()[1]) * 1024
    except Exception:
        pass
    import oracle

    def explicit_bytes(N, lx, ly):
        nn, nnn = oracle.bond_pairs(oracle.SQUARE2D, N, lx, ly)
        dim = math.comb(N, N // 2)
        nnz = dim * (1 + kbar(N, N // 2, list(map(tuple, nn)) + list(map(tuple, nnn))))
        return 24 * nnz + 8 * (dim + 1)
    sizes = {'N=24 4x6': explicit_bytes(24, 4, 6), 'N=28 4x7': explicit_bytes(28, 4, 7),
             'N=30 6x5': explicit_bytes(30, 6, 5)}
    return {'cpu_model': model, 'logical_cores': os.cpu_count(), 'ram_bytes': ram,
            'explicit_matrix_bytes': {k: int(v) for k, v in sizes.items()},
            'explicit_matrix_fits_ram': {k: (bool(ram and v < 0.8 * ram) if ram else None) for k, v in sizes.items()}}


class CpuSolve:
    """One full CPU Krylov-Schur eigensolve by the oracle port on all host
    threads: the explicit matrix in the reference layout (int64 columns,
    complex128 values, rows sorted as PETSc AIJ keeps them) and the
    Krylov-Schur restatement in complex128, with the workload's nev, ncv,
    tolerance and start vector.  The matrix build is setup (as the device
    run's is) and timed separately.  A few extra SpMVs split the solve's time
    per step into the SpMV and the rest (orthogonalisation, restarts), which
    is what the extrapolation to a larger basis scales."""

    def __init__(self, wl, size=None):
        import oracle
        self.wl = wl
        ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
        self.cfg = (N, mag, nev, ncv, tol, J1, D1, J2, D2)
        self.lt = oracle.SQUARE2D if ltype == 'square2D' else oracle.CHAIN1D
        if size is None:
            size = CPU_SAMPLE.get(wl, (N, lx, ly))
        self.sN, self.slx, self.sly = size
        t0 = time.perf_counter()
        self.M = oracle.Model(self.lt, self.sN, self.slx, self.sly, mag, J1, D1, J2, D2)
        self.nnz = self.M.build(3)
        self.t_build = time.perf_counter() - t0
        self.dim = self.M.dim

    def run(self):
        import numpy as np
        import oracle
        N, mag, nev, ncv, tol, J1, D1, J2, D2 = self.cfg
        t0 = time.perf_counter()
        r = self.M.eps_solve(nev=nev, ncv=ncv, tol=tol, seed=0, vectors=False)
        t_solve = time.perf_counter() - t0
        x = oracle.start_vector(1, self.dim)
        reps, t0 = 0, time.perf_counter()
        while reps < 3 or (reps < 20 and time.perf_counter() - t0 < 1.0):
            self.M.apply(x)
            reps += 1
        t_spmv = (time.perf_counter() - t0) / reps
        return {'N': self.sN, 'lattice': '%dx%d' % (self.slx, self.sly), 'dim': self.dim, 'nnz': self.nnz,
                'build_s': self.t_build, 'solve_s': t_solve, 'nhv': r['nhv'], 'its': r['its'],
                'nconv': r['nconv'], 'eigenvalues': [float(e) for e in np.sort(r['evals'])[:nev]],
                'spmv_s': t_spmv, 'threads': oracle.get_threads()}


def cpu_extrapolate(meas, wl, nhv):
    """Seconds of the CPU solve of workload wl, from a measured solve of a
    smaller member of the family: per step, the SpMV scales with the stored
    entries and the rest with the basis size; times the H.v count nhv."""
    ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    import oracle
    lt = oracle.SQUARE2D if ltype == 'square2D' else oracle.CHAIN1D
    nn, nnn = oracle.bond_pairs(lt, N, lx, ly)
    pairs = list(map(tuple, nn)) + (list(map(tuple, nnn)) if J2 else [])
    dim = math.comb(N, mag + N // 2)
    nnz = dim * (1 + kbar(N, mag + N // 2, pairs))
    per_step = meas['solve_s'] / max(meas['nhv'], 1)
    other = max(0.0, per_step - meas['spmv_s'])
    t = nhv * (meas['spmv_s'] * nnz / meas['nnz'] + other * dim / meas['dim'])
    note = ('measured N=%d %s CPU solve (%.2f s, %d H.v, %.4f s per SpMV) scaled per step to N=%d: SpMV by stored '
            'entries (x%.2f), orthogonalisation by basis size (x%.2f); times %d H.v'
            % (meas['N'], meas['lattice'], meas['solve_s'], meas['nhv'], meas['spmv_s'], N, nnz / meas['nnz'],
               dim / meas['dim'], nhv))
    return t, note


def run_reference(args):
    """The reference's CPU path (the oracle port: explicit matrix in the
    reference layout, Krylov-Schur in complex128) on all host threads.  Each
    step is one full CPU solve of the largest family member that fits
    (N=24 4x6 for the N=30 workload), timed end to end; the line's value
    extrapolates it to the workload (kind 'port-extrapolated').  Steps are
    capped at 2 solves so the run stays within a few minutes; warm-up solves
    are not run (the matrix build, untimed, touches all memory first)."""
    ws, rk, lr = _rank_info()
    if rk != 0:
        return 0
    wl = args.workload
    ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    size = None
    if getattr(args, 'cpu_size', None):
        size = tuple(int(v) for v in args.cpu_size.split(','))
    cs = CpuSolve(wl, size)
    nrun = max(1, min(args.steps, 2))
    runs = [cs.run() for _ in range(nrun)]
    meas = dict(runs[-1])
    meas['solve_s'] = sum(r['solve_s'] for r in runs) / nrun
    meas['solve_s_each'] = [r['solve_s'] for r in runs]
    if (cs.sN, cs.slx, cs.sly) == (N, lx, ly):
        v, kind, note = meas['solve_s'], 'port', 'full CPU eigensolve of the workload itself'
    else:
        v, note = cpu_extrapolate(meas, wl, NHV_DEVICE.get(wl, meas['nhv']))
        kind = 'port-extrapolated'
        note += ' (the H.v count of the device solve of this workload from the same start vector)'
    cpu = {'value': v, 'unit': 's', 'cores': meas['threads'], 'kind': kind, 'sample': note,
           'measured': meas, 'host': host_info()}
    line = {'metric': METRIC, 'value': v, 'unit': 's', 'n_gpus': args.gpus, 'steps': nrun, 'warmup': 0,
            'ms_per_step': v * 1e3, 'higher_is_better': False, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'c128', 'data': 'synthetic',
            'config': workload_config(wl), 'impl': 'reference', 'cpu_baseline': cpu,
            'timed_region_s': sum(r['solve_s'] for r in runs),
            'e2e': {'value': v, 'unit': 's', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line, default=_json_default))
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


C3 = dict(N=20, J1=1.0, J2=0.2, W=2.0, nev=2, ncv=16, tol=1e-9)


def disorder_sweep(ed, env, seeds, restart='auto', plain_sample=16):
    """C3: disorder sweep, chain N=20 (J1=1, J2=0.2, Delta=1), h_i ~ U[-2, 2]
    from mt19937_64(seed) (RandomDisorder::hi_init with srand_seq[k] = seed),
    Sz = 0, 1, 2, lowest 2 pairs at eps_tol 1e-9.  Batched: one batch per
    sector over all `seeds`, the three sectors solved at once (solve_batches:
    one environment, host thread and stream per sector; expansion sweeps
    replayed from CUDA graphs), timed on the host around the call; the same
    batches one sector after another, and at once with direct launches, are
    timed beside it.  Plain: the same solves one at a time
    for `plain_sample` seeds per sector spread over the whole seed range
    (every restart tile of the batch), timed per solve, eigenvalues checked
    against the batch at 1e-8."""
    import numpy as np
    import torch
    N, J1, J2, W, nev, ncv, tol = (C3[k] for k in ('N', 'J1', 'J2', 'W', 'nev', 'ncv', 'tol'))
    fields = np.stack([ed.random_fields(sd, N, -W, W) for sd in seeds])
    sectors = (0, 1, 2)
    hams, envs = {}, {}
    for mag in sectors:  # one environment (stream) per sector: the sectors can run at once
        env = envs[mag] = ed.Environment(nspins=N, device=torch.cuda.current_device())
        b = ed.Basis(env, mag)
        h = ed.Hamiltonian(env, b, ed.chain1D(env), J1, 1.0, J2, J2)
        h.build_diag(env)
        h.build_off_diag(env)
        hams[mag] = (b, h)
    for mag in sectors:  # warm-up on a small batch per sector
        bt = ed.DisorderBatch(hams[mag][1], fields[:8])
        bt.solve(nev=nev, ncv=ncv, tol=tol, seed=0)
        del bt
    torch.cuda.synchronize()
    brestart = restart if restart in ('auto', 'fp64', 'pair') else 'auto'
    kcount = lambda: sum(e.kernel_count() for e in envs.values())

    def batched(concurrent, graphs=False):
        bts = []
        for mag in sectors:
            bt = ed.DisorderBatch(hams[mag][1], fields)
            bt.set_restart_arithmetic(brestart)
            bt.set_graphs(graphs)
            bts.append(bt)
        torch.cuda.synchronize()
        k0 = kcount()
        t0 = time.perf_counter()
        if concurrent:  # the three sectors at once, one host thread and stream each
            rs = ed.solve_batches(bts, nev=nev, ncv=ncv, tol=tol, seed=0)
        else:
            rs = [bt.solve(nev=nev, ncv=ncv, tol=tol, seed=0) for bt in bts]
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        return t, kcount() - k0, rs, [list(bt.hv_tile()) for bt in bts]

    t_seq, _, rs_seq, _ = batched(False, graphs=True)
    t_direct, _, rs_direct, _ = batched(True, graphs=False)
    t_batch, launches, rs, tiles = batched(True, graphs=True)
    max_err = max(float(r['errs'].max()) for r in rs)
    bad = sum(int((r['nconv'] < nev).sum()) for r in rs)
    its = [r['its'] for r in rs]
    batch_evals = {mag: r['evals'] for mag, r in zip(sectors, rs)}
    same_seq = all(np.allclose(a['evals'], b['evals'], rtol=1e-12, atol=0) for a, b in zip(rs, rs_seq))
    nplain = min(plain_sample, len(seeds))
    pick = sorted(set(np.linspace(0, len(seeds) - 1, nplain).round().astype(int).tolist()))
    t0 = time.perf_counter()
    agree = True
    perr = 0.0
    for mag in sectors:
        b, _ = hams[mag]
        env = envs[mag]
        for k in pick:
            h = ed.Hamiltonian(env, b, ed.chain1D(env), J1, 1.0, J2, J2)
            h.build_diag(env)
            h.build_off_diag(env)
            h.build_disorder(env, fields[k])
            eps = ed.Solver.SolverInit(h, nev, ncv)
            ed.Solver.EPSSetTolerances(eps, tol)
            eps.set_restart_arithmetic(restart)
            ed.Solver.solve(env, eps)
            for i in range(nev):
                e, er = ed.Solver.eigenvalue(eps, i)
                perr = max(perr, er)
                agree &= abs(e - batch_evals[mag][k][i]) <= 1e-8 * abs(e)
            ed.Solver.SolverClean(eps)
    torch.cuda.synchronize()
    t_plain = (time.perf_counter() - t0) / (len(pick) * len(sectors))
    nsolve = len(seeds) * len(sectors)
    return {'batched_samples_per_s': nsolve / t_batch, 'plain_samples_per_s': 1.0 / t_plain,
            'batched_over_plain': (nsolve / t_batch) * t_plain, 'batched_seconds': t_batch, 'solves': nsolve,
            'sectors_at_once': True, 'batched_one_sector_at_a_time_samples_per_s': nsolve / t_seq,
            'cuda_graphs': True, 'batched_direct_launches_samples_per_s': nsolve / t_direct,
            'direct_launches_eigenvalues_agree_1e-12': bool(all(np.allclose(a['evals'], b['evals'], rtol=1e-12, atol=0)
                                                              for a, b in zip(rs, rs_direct))),
            'eigenvalues_agree_with_one_sector_at_a_time_1e-12': bool(same_seq),
            'max_rel_residual': max_err, 'plain_max_rel_residual': perr, 'unconverged': bad,
            'restarts_per_sector': its, 'gpu_launches': launches, 'restart_arithmetic': restart,
            'hv_tile_per_sector': tiles,
            'plain_sample': '%d seeds per sector (indices %s), one solve at a time' % (len(pick), pick),
            'eigenvalues_agree_1e-8': bool(agree), 'fields': fields, 'batch_evals': batch_evals,
            'config': 'chain1D N=20 J1=1 J2=0.2 Delta=1, h_i~U[-2,2] seeds %d..%d, Sz=0,1,2, nev=2, ncv=16, '
                      'eps_tol=1e-9, dims %s' % (seeds[0], seeds[-1], [b.size for b, _ in hams.values()])}


def run_disorder(args):
    """C3 as its own line: samples/s of the batched sweep over the 1,536
    solves, the plain one-at-a-time rate beside it, and a CPU baseline from
    the oracle port on a bounded subset.  Under torchrun the seeds are split
    over the ranks (no data-path collective; host scalars reduced)."""
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
    nseeds = args.seeds
    mine = shard_units(nseeds, rk, ws)
    if ws > 1:
        torch.distributed.barrier()
    r = disorder_sweep(ed, None, mine, args.restart, args.plain_sample)
    t_batch = dist_reduce(r['batched_seconds'], ws, 'max')
    max_err = dist_reduce(r['max_rel_residual'], ws, 'max')
    bad = int(dist_reduce(r['unconverged'], ws, 'sum'))
    nsolve = nseeds * 3
    if rk != 0:
        return 0
    N, J1, J2, nev, tol = C3['N'], C3['J1'], C3['J2'], C3['nev'], C3['tol']
    cpu = None
    if not args.no_cpu:
        try:
            k = max(1, min(args.cpu_seeds, len(mine)))
            sps, cores, cev = c3_cpu_sample(r['fields'][:k], (0, 1, 2), N, J1, J2, nev, tol)
            cagree = all(abs(cev[mag][i][q] - r['batch_evals'][mag][i][q]) <= 1e-8 * abs(cev[mag][i][q])
                         for mag in (0, 1, 2) for i in range(k) for q in range(nev))
            cpu = {'value': sps, 'unit': 'samples/s', 'cores': cores, 'kind': 'port',
                   'sample': '%d seeds x 3 sectors: full CPU eigensolves (explicit CSR build + Krylov-Schur, '
                             'nev=2, tol 1e-9), the rate extrapolated to the sweep' % k,
                   'eigenvalues_agree_1e-8': bool(cagree)}
        except Exception as ex:  # reported, never fatal
            cpu = {'value': None, 'unit': 'samples/s', 'cores': None, 'kind': 'port', 'sample': 'failed: %s' % ex}
    out = {k: v for k, v in r.items() if k not in ('fields', 'batch_evals', 'config')}
    out.update(batched_seconds=t_batch, max_rel_residual=max_err, unconverged=bad,
               batched_samples_per_s=nsolve / t_batch)
    line = {'metric': METRIC, 'workload': 'c3', 'value': nsolve / t_batch, 'unit': 'samples/s',
            'higher_is_better': True, 'n_gpus': ws, 'steps': 1, 'warmup': args.warmup,
            'scaling': 'strong',  # the 1,536 solves are split over the ranks by seed
            'batched': out, 'cpu_baseline': cpu, 'dtype': 'f64', 'data': 'synthetic',
            'dtype_note': DTYPE_NOTE,
            'config': {'workload': 'c3 ' + r['config'].replace('seeds 0..', 'seeds 0..')}}
    print(json.dumps(line, default=_json_default))
    return 0


C4 = {'4x4': (16, 4, 4), '4x6': (24, 4, 6)}


def gradient_timing(ed, restart='auto', seed=71):
    """C4: adjoint gradients on the 4x4 and 4x6 J1-J2 lattices (J2 = 0.5,
    Delta = 1) with per-bond couplings J_b = base_b (1 + 0.1 z_b),
    z_b ~ N(0, 1) from mt19937_64(seed), D_b = J_b, and fields
    h_i ~ U[-0.5, 0.5] from mt19937_64(seed + 1).  Timed on the host (each
    step returns host results): the solve (nev=4, tol 1e-12), the
    Hellmann-Feynman gradient of E0 and of the lowest-4 sum, and the adjoint
    (MINRES, tol 1e-8, at most 4000 iterations) gradient of <S_0.S_far>.  One bond and one field derivative of
    E0 are checked against central differences (step 1e-5) of device
    energies."""
    import numpy as np
    import torch
    out = {}
    for name, (N, lx, ly) in C4.items():
        env = ed.Environment(nspins=N)
        b = ed.Basis(env, 0)
        lat = ed.square2D(env, lx, ly)
        pairs = np.concatenate([lat.nn_pairs, lat.nnn_pairs])
        z = ed.random_normal(seed, len(pairs))
        J = np.where(np.arange(len(pairs)) < len(lat.nn_pairs), 1.0, 0.5) * (1 + 0.1 * z)
        D = J.copy()
        hi = ed.random_fields(seed + 1, N, -0.5, 0.5)

        def solve(Jx, Dx, hx, nev=4):
            h = ed.Hamiltonian.from_bonds(env, b, pairs, Jx, Dx)
            h.build_diag(env)
            h.build_off_diag(env)
            h.build_disorder(env, hx)
            eps = ed.Solver.SolverInit(h, nev, 20)
            ed.Solver.EPSSetTolerances(eps, 1e-12)
            eps.set_restart_arithmetic(restart)
            ed.Solver.solve(env, eps)
            return h, eps
        solve(J, D, hi)  # warm-up (run-time compiled kernels, allocations)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h, eps = solve(J, D, hi)
        e = [ed.Solver.eigenvalue(eps, n)[0] for n in range(4)]
        t_solve = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, v0, _ = ed.Solver.solution(eps, 0)
        dJ, dD, dh = ed.Adjoint.energy_gradient(b, pairs, v0)
        t_e0 = time.perf_counter() - t0
        t0 = time.perf_counter()
        sJ, sD, sh = ed.Adjoint.eigenvalue_sum_gradient(eps, pairs, 4)
        t_sum = time.perf_counter() - t0
        far = (lx // 2) * ly + ly // 2
        obs = [(1.0, ed.Adjoint.SISJ, 0, far)]
        t0 = time.perf_counter()
        val, cJ, cD, ch, info = ed.Adjoint.expectation_gradient(h, pairs, e[0], v0, obs, tol=1e-8, max_it=4000)
        t_corr = time.perf_counter() - t0
        ed.Solver.SolverClean(eps)
        d = 1e-5

        def e0(Jx, Dx, hx):
            _, ep = solve(Jx, Dx, hx, nev=1)
            v = ed.Solver.eigenvalue(ep, 0)[0]
            ed.Solver.SolverClean(ep)
            return v
        # J_q and D_q together (Delta = 1 ties them): dE0/dJ_q + dE0/dD_q
        q = len(pairs) // 3
        Jp, Jm = J.copy(), J.copy()
        Jp[q] += d
        Jm[q] -= d
        fdJ = (e0(Jp, Jp, hi) - e0(Jm, Jm, hi)) / (2 * d)
        hp, hm = hi.copy(), hi.copy()
        hp[1] += d
        hm[1] -= d
        fdh = (e0(J, D, hp) - e0(J, D, hm)) / (2 * d)
        out[name] = {'N': N, 'dim': b.size, 'bonds': len(pairs), 'solve_s': t_solve, 'grad_e0_s': t_e0,
                     'grad_sum4_s': t_sum, 'grad_corr_minres_s': t_corr, 'minres_its': info['its'],
                     'minres_relres': info['relres'], 'E': e, 'S0_Sfar': val,
                     'fd_check': {'bond': q, 'dE0_dJ': float(dJ[q] + dD[q]), 'fd': fdJ,
                                  'rel_err': abs(fdJ - dJ[q] - dD[q]) / max(1.0, abs(fdJ)),
                                  'site': 1, 'dE0_dh': float(dh[1]), 'fd_h': fdh,
                                  'rel_err_h': abs(fdh - dh[1]) / max(1.0, abs(fdh))}}
    return out


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


def run_sisj_only(args):
    """Time the all-pairs <S_i.S_j> and <S^z_i S^z_j> measurements alone on a
    seeded random real state of the workload's sector (the solver's
    eigenvectors are real): K calls after W warm-up calls, each call all N^2
    pairs (N (N + 1) / 2 evaluated, the rest mirrored)."""
    import numpy as np
    import torch
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300 as ed
    wl = args.workload
    ltype, N, lx, ly, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    env = ed.Environment(nspins=N)
    b = ed.Basis(env, mag)
    g = torch.Generator(device='cuda')
    g.manual_seed(5)
    psi = torch.randn(b.size, dtype=torch.float64, device='cuda', generator=g)
    psi /= torch.linalg.vector_norm(psi)
    psi = psi.to(torch.complex128)
    out = {'mode': 'sisj-only', 'workload': wl, 'dim': b.size, 'pairs': N * N, 'evaluated': N * (N + 1) // 2}
    for name, cls in (('SiSj', ed.SiSj), ('SzSz', ed.SzSz)):
        corr = cls(env, b)
        for _ in range(args.warmup):
            corr.AllPairs(psi)
        torch.cuda.synchronize()
        k0 = env.kernel_count()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            C = corr.AllPairs(psi)
        torch.cuda.synchronize()
        sec = (time.perf_counter() - t0) / args.steps
        out[name] = {'s_per_all_pairs': sec, 'launches_per_call': (env.kernel_count() - k0) / args.steps,
                     'trace': float(np.real(np.trace(C))), 'c01': float(np.real(C[0, 1]))}
    # one FP64 FMA per evaluated off-diagonal pair and basis state (the flip part)
    offd = N * (N - 1) // 2
    out['SiSj']['fp64_fma_per_s'] = offd * b.size / out['SiSj']['s_per_all_pairs']
    print(json.dumps(out))
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
        # a user allocates pinned buffers once and reuses them: their one-time
        # first-transfer cost (about 0.1 s per 2.5 GB here) is paid before the
        # timed region by one untimed copy each way
        warm = torch.empty(dim, dtype=torch.complex128, device='cuda')
        warm.copy_(start_host, non_blocking=True)
        for o in out_host:
            o.copy_(warm, non_blocking=True)
        torch.cuda.synchronize()
        del warm
        t0 = time.perf_counter()
        phases = {}

        def mark(key, t_prev):
            torch.cuda.synchronize()
            t_now = time.perf_counter()
            phases[key] = t_now - t_prev
            return t_now
        b2 = ed.Basis(env, mag)
        tm = mark('basis_s', t0)
        lat2 = ed.square2D(env, lx, ly) if ltype == 'square2D' else ed.chain1D(env)
        H2 = ed.Hamiltonian(env, b2, lat2, J1, D1, J2, D2)
        H2.build_diag(env)
        H2.build_off_diag(env)
        tm = mark('hamiltonian_s', tm)
        eps2 = ed.Solver.SolverInit(H2, nev, ncv if ncv else ed.PETSC_DEFAULT)
        ed.Solver.EPSSetTolerances(eps2, tol, 0)
        eps2.set_restart_arithmetic(args.restart)
        tm = mark('solver_init_s', tm)
        eps2.set_initial_vector(start_host)
        tm = mark('upload_s', tm)
        phases['setup_and_upload_s'] = tm - t0
        ed.Solver.solve(env, eps2)
        torch.cuda.synchronize()
        phases['solve_s'] = time.perf_counter() - t0 - phases['setup_and_upload_s']
        vals2 = []
        tm = time.perf_counter()
        for i in range(nev):
            e, err = ed.Solver.eigenvalue(eps2, i)
            vals2.append(e)
            ed.Solver.solution_host(eps2, i, out=out_host[i])
            tm = mark('readback_vec%d_s' % i, tm)
        torch.cuda.synchronize()
        t_e2e = time.perf_counter() - t0
        phases['readback_s'] = t_e2e - phases['setup_and_upload_s'] - phases['solve_s']
        ed.Solver.SolverClean(eps2)
        del H2, b2
        e2e = {'value': t_e2e, 'unit': 's', 'h2d_bytes_per_step': int(16 * dim + 8 * 2 * len(pairs)),
               'd2h_bytes_per_step': int(16 * dim * nev), 'steps': 1, 'phases': phases,
               'host_buffers': 'pinned, allocated and used once by an untimed copy before the timed region',
               'eigenvalues_match_device_run': bool(np.allclose(vals2, evals, rtol=1e-10, atol=0))}

    # the same solve at the largest size the reference's CPU path can hold,
    # on the device and on the host cores (both measured in this run)
    cpu = None
    same = None
    c3 = c4 = None
    t_cpu = time.perf_counter()
    if rk == 0 and not args.no_cpu:
        try:
            cs = CpuSolve(wl)
            meas = cs.run()
            if (cs.sN, cs.slx, cs.sly) == (N, lx, ly):
                cpu = {'value': meas['solve_s'], 'unit': 's', 'cores': meas['threads'], 'kind': 'port',
                       'sample': 'full CPU eigensolve of the workload itself', 'measured': meas}
            else:
                v, note = cpu_extrapolate(meas, wl, st['nhv'])
                cpu = {'value': v, 'unit': 's', 'cores': meas['threads'], 'kind': 'port-extrapolated',
                       'sample': note + ' (the H.v count of this run\'s device solve)', 'measured': meas}
                gs = device_solve_seconds(ed, env, cs.sN, cs.slx, cs.sly, wl, args.restart)
                same = {'N': cs.sN, 'lattice': '%dx%d' % (cs.slx, cs.sly), 'gpu_solve_s': gs['seconds'],
                        'gpu_nhv': gs['nhv'], 'cpu_solve_s': meas['solve_s'], 'cpu_nhv': meas['nhv'],
                        'cpu_cores': meas['threads'], 'cpu_over_gpu': meas['solve_s'] / gs['seconds'],
                        'eigenvalues_agree_1e-10': bool(np.allclose(gs['eigenvalues'], meas['eigenvalues'],
                                                                    rtol=1e-10, atol=0))}
            cpu['host'] = host_info()
        except Exception as ex:  # reported, never fatal
            cpu = {'value': None, 'unit': 's', 'cores': None, 'kind': 'port', 'sample': 'failed: %s' % ex}
    sections = {'cpu_baseline_and_same_size_s': time.perf_counter() - t_cpu}
    rates = None
    if rk == 0:
        try:
            rates = env.probe_rates()
        except Exception as ex:
            rates = {'failed': str(ex)}
    if rk == 0 and wl == 'c5' and not args.no_extra:
        t0 = time.perf_counter()
        try:
            c3 = disorder_sweep(ed, env, list(range(args.seeds)), args.restart, args.plain_sample)
            c3 = {k: v for k, v in c3.items() if k not in ('fields', 'batch_evals')}
        except Exception as ex:
            c3 = {'failed': str(ex)}
        sections['c3_s'] = time.perf_counter() - t0
        t0 = time.perf_counter()
        try:
            c4 = gradient_timing(ed, args.restart)
        except Exception as ex:
            c4 = {'failed': str(ex)}
        sections['c4_s'] = time.perf_counter() - t0

    if rk != 0:
        return 0
    line = {
        'metric': METRIC, 'value': ms_step / 1e3, 'unit': 's', 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_step, 'higher_is_better': False, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': workload_config(wl),
        'dtype_note': DTYPE_NOTE if args.restart != 'pair' else DTYPE_NOTE + '; restart products as float pairs '
                      'on the FP32 units (requested: error below 2^-45 per product)',
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
        'clocks': clocks, 'cpu_baseline': cpu, 'same_size_gpu_vs_cpu': same, 'c3': c3, 'c4': c4,
        'unit_rates': rates, 'bench_sections_s': sections,
    }
    print(json.dumps(line, default=_json_default))
    return 0


def _json_default(o):
    """numpy scalars and arrays in the JSON line."""
    import numpy as np
    if isinstance(o, np.ndarray):
        return o.tolist()
    if isinstance(o, np.generic):
        return o.item()
    raise TypeError('not JSON serializable: %r' % type(o))


def device_solve_seconds(ed, env_unused, N, lx, ly, wl, restart, reps=3):
    """Device-resident solve of the workload's family member N (lx x ly) with
    the workload's nev / ncv / tol: one warm-up solve, then the mean of
    `reps` solves timed with CUDA events on the current stream."""
    import torch
    ltype, _, _, _, J1, D1, J2, D2, mag, nev, ncv, tol = WORKLOADS[wl]
    env = ed.Environment(nspins=N)
    b = ed.Basis(env, mag)
    lat = ed.square2D(env, lx, ly) if ltype == 'square2D' else ed.chain1D(env)
    H = ed.Hamiltonian(env, b, lat, J1, D1, J2, D2)
    H.build_diag(env)
    H.build_off_diag(env)

    def one():
        eps = ed.Solver.SolverInit(H, nev, ncv if ncv else ed.PETSC_DEFAULT)
        ed.Solver.EPSSetTolerances(eps, tol, 0)
        eps.set_restart_arithmetic(restart)
        ed.Solver.solve(env, eps)
        return eps
    ed.Solver.SolverClean(one())
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(reps):
        eps = one()
        if k < reps - 1:
            ed.Solver.SolverClean(eps)
    e1.record(stream)
    torch.cuda.synchronize()
    st = eps.stats()
    ev = sorted(ed.Solver.eigenvalue(eps, i)[0] for i in range(min(nev, st['nreported'])))
    ed.Solver.SolverClean(eps)
    return {'seconds': e0.elapsed_time(e1) / 1e3 / reps, 'nhv': st['nhv'], 'eigenvalues': ev}


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
    ap.add_argument('--restart', default='auto', choices=('auto', 'fp64', 'pair', 'fixed', 'exact'),
                    help='restart-combination products of the real-storage solve (auto: the fastest form with every '
                         'product FP64 or better; fp64: FP64 beside exact integers; fixed: 56-bit fixed point on the '
                         'integer units; pair: float pairs on the FP32 units; exact: tensor-core slices)')
    ap.add_argument('--no-extra', action='store_true', help='skip the C3 / C4 sub-objects of the default line')
    ap.add_argument('--probe-rates', action='store_true',
                    help='print the measured FP64 FMA / FP64 mma / FP16-FP32 mma rates and exit')
    ap.add_argument('--cpu-size', default=None,
                    help='N,lx,ly of the measured CPU solve (default: the largest family member that fits)')
    ap.add_argument('--real-storage', action='store_true',
                    help='--hv-only on real vectors in real storage (float64, as inside the solve)')
    ap.add_argument('--variant', default='auto', help='--hv-only: force an H.v launch variant (default: autotuner)')
    ap.add_argument('--hv-only', action='store_true', help='time the H.v kernel alone')
    ap.add_argument('--sisj-only', action='store_true',
                    help='time the all-pairs <S_i.S_j> / <S^z_i S^z_j> measurements alone on a random real state')
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
    if args.sisj_only:
        return run_sisj_only(args)
    if args.probe_rates:
        from lsquantumed_gb300.build import build
        build()
        import lsquantumed_gb300 as ed
        print(json.dumps(ed.Environment(nspins=2).probe_rates()))
        return 0
    if args.workload == 'c3':
        return run_disorder(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
