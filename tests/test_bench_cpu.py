"""CPU checks of the benchmark's byte accounting: k-bar (mean off-diagonal
entries per row) for every workload from the reference's bond tables, and the
algorithmic bytes per H.v row that roofline.achieved is computed from."""
import importlib.util
import os

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def bench():
    spec = importlib.util.spec_from_file_location('bench_under_test', os.path.join(ROOT, 'bench.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _pairs(ltype, N, lx, ly, with_nnn):
    nn, nnn = oracle.bond_pairs(ltype, N, lx, ly)
    pairs = [tuple(p) for p in nn]
    if with_nnn:
        pairs += [tuple(p) for p in nnn]
    return pairs


@pytest.mark.parametrize('case,B', [
    ((oracle.SQUARE2D, 30, 6, 5, True), 120),   # N=30 6x5 J1-J2: k-bar 62.07
    ((oracle.SQUARE2D, 20, 4, 5, True), 80),    # 4x5 J1-J2: 42.1
    ((oracle.CHAIN1D, 16, 1, 16, False), 16),   # chain N=16: 8.53
    ((oracle.CHAIN1D, 20, 1, 20, True), 40),    # chain N=20 J1-J2 (disorder sweep): 21.05
    ((oracle.SQUARE2D, 16, 4, 4, True), 64),    # 4x4 J1-J2: 34.1
    ((oracle.SQUARE2D, 24, 4, 6, True), 96),    # 4x6 J1-J2: 50.1
])
def test_kbar_from_reference_bonds(bench, case, B):
    """k-bar = B N / (2 (N - 1)) at Sz=0 for B distinct bonds."""
    ltype, N, lx, ly, nnn = case
    kb = bench.kbar(N, N // 2, _pairs(ltype, N, lx, ly, nnn))
    assert abs(kb - B * N / (2 * (N - 1))) < 1e-12, kb


def test_bytes_per_row(bench):
    kb = bench.kbar(30, 15, _pairs(oracle.SQUARE2D, 30, 6, 5, True))
    # real storage (the solve): 8 x_s + 8 k-bar + 8 y_s + 4 state + 8 diagonal
    assert abs(bench.hv_bytes_per_row(kb, 'real_storage') - (28 + 8 * kb)) < 1e-9
    assert abs(bench.hv_bytes_per_row(kb, 'real_storage') - 524.55) < 0.01
    # complex128 vectors and 16-byte gathers
    assert abs(bench.hv_bytes_per_row(kb, 'complex') - 1037.1) < 0.05
    # one launch at N=30 moves 81.4 GB of algorithmic bytes
    assert abs(bench.hv_bytes_per_row(kb, 'real_storage') * 155117520 / 1e9 - 81.4) < 0.05


def test_c3_cpu_sample(bench):
    """The disorder-sweep CPU baseline solves what the batched sweep solves:
    the chain J1-J2 with the realisation's fields, in each sector; its lowest
    levels match dense diagonalisation."""
    import numpy as np
    N, nev = 12, 2
    fields = [oracle.rd_hi(s, N, -2.0, 2.0) for s in (0, 1)]
    sps, cores, ev = bench.c3_cpu_sample(fields, (0, 1), N, 1.0, 0.2, nev, 1e-10)
    assert sps > 0 and cores >= 1
    for mag in (0, 1):
        for hi, got in zip(fields, ev[mag]):
            M = oracle.Model(oracle.CHAIN1D, N, 1, N, mag, 1.0, 1.0, 0.2, 0.2)
            M.build(3, hi)
            want = np.linalg.eigvalsh(M.dense())[:nev]
            assert np.allclose(got, want, rtol=1e-10, atol=0), (mag, got, want)


def test_reference_arm_json_contract():
    """`bench.py --impl reference` (the oracle port on the host cores: full CPU
    eigensolves of a smaller member of the workload's family, here the 4x4
    lattice to keep the test short) prints one JSON line with the same metric
    and workload as the GPU arm, impl "reference", steps = the solves it
    actually ran, a cpu_baseline that carries the measured solve and labels
    the extrapolated value, and an e2e entry with no host-device bytes."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '5',
                        '--warmup', '3', '--cpu-size', '16,4,4'], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line['impl'] == 'reference'
    assert line['unit'] == 's' and line['higher_is_better'] is False
    assert line['config']['workload'].startswith('c5 ') and line['config']['dim'] == 155117520
    assert line['steps'] == 2 and line['warmup'] == 0  # solves actually run (capped at 2)
    cb = line['cpu_baseline']
    assert cb['kind'] == 'port-extrapolated' and cb['cores'] >= 1 and cb['value'] == line['value'] > 0
    m = cb['measured']
    assert m['N'] == 16 and m['dim'] == 12870 and m['nhv'] > 0 and len(m['solve_s_each']) == 2
    assert abs(line['timed_region_s'] - sum(m['solve_s_each'])) < 1e-9
    assert cb['host']['logical_cores'] >= 1
    assert line['e2e'] == {'value': line['value'], 'unit': 's', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}


def test_cpu_extrapolation_model(bench):
    """The N=30 estimate scales the measured per-step SpMV by stored entries
    and the rest of the step by basis size, times the H.v count."""
    meas = {'N': 24, 'lattice': '4x6', 'dim': 2704156, 'nnz': 137980548, 'solve_s': 30.0, 'nhv': 300,
            'spmv_s': 0.06}
    t, note = bench.cpu_extrapolate(meas, 'c5', 334)
    dim30 = 155117520
    nnz30 = dim30 * (1 + 120 * 30 / (2 * 29))
    want = 334 * (0.06 * nnz30 / meas['nnz'] + 0.04 * dim30 / meas['dim'])
    assert abs(t - want) <= 1e-9 * want
    assert 'times 334 H.v' in note


def test_host_info(bench):
    info = bench.host_info()
    assert info['logical_cores'] >= 1
    sizes = info['explicit_matrix_bytes']
    # N=30 6x5: 155M rows x (1 + 62.07) entries x 24 B = 235 GB
    assert 230e9 < sizes['N=30 6x5'] < 240e9
    assert 3.0e9 < sizes['N=24 4x6'] < 3.6e9
