"""The drop-in driver (lsqed_main, the reference's examples/main.cpp on the
lsqed.hpp shim) against the oracle: ground-state energy line, magAF, and the
dsf_d0.dat file (reference layout, phys.tmpl_func.hpp:126-200) whose energies
E_n - E0 must be levels of the spectrum.

Tolerances: E0 to the 6 decimals the reference's "%12f" prints; magAF to
1e-9 (printed with 10 decimals); DSF energies to 1e-10 (printed "%.13e").
"""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from oracle import Model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def driver():
    from lsquantumed_gb300.build import build, DRIVER
    build()
    return DRIVER


def test_driver_chain12(driver, tmp_path):
    N, nev_dsf = 12, 4
    r = subprocess.run([driver, '-n', str(N), '-ltype', 'chain1D', '-j1', '1', '-d1', '1', '-j2', '0.3', '-d2', '0.3',
                        '-eps_tol', '1e-11', '-dsf_nev', str(nev_dsf), '-path', str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    M = Model(oracle.CHAIN1D, N, 1, N, 0, 1.0, 1.0, 0.3, 0.3)
    M.build(3)
    w, V = np.linalg.eigh(M.dense())
    # ground-state line: "  0     <E0>       <err>"
    m = re.search(r'^\s+0\s+(-?\d+\.\d+)\s+(\S+)\s*$', r.stdout, re.M)
    assert m, r.stdout
    assert abs(float(m.group(1)) - w[0]) <= 1e-6
    assert float(m.group(2)) <= 1e-8
    # magAF of the ground state (non-degenerate for this chain)
    assert w[1] - w[0] > 1e-3
    psi = V[:, 0].astype(np.complex128)
    want = oracle.squared_sublatt_mag_af(M, oracle.sublattice_af(oracle.CHAIN1D, N), psi).real
    m = re.search(r'^magAF: (\S+)$', r.stdout, re.M)
    assert m and abs(float(m.group(1)) - want) <= 1e-9, (m, want)
    # dsf_d0.dat: header, then N blocks of nev lines "dE  Re c"
    lines = open(os.path.join(str(tmp_path), 'dsf_d0.dat')).read().splitlines()
    assert lines[0].startswith('#------------------------------- Parameters')
    assert re.match(r'^#\s+nspins:\s+12\s*$', lines[1])
    rows = [ln for ln in lines if not ln.startswith('#')]
    assert len(rows) == N * nev_dsf
    assert sum(1 for ln in lines if ln.startswith('# spin:')) == N
    dE = np.array([float(ln.split()[0]) for ln in rows[:nev_dsf]])
    assert abs(dE[0]) <= 1e-10
    for d in dE:
        assert np.min(np.abs((w - w[0]) - d)) <= 1e-10, (d, w[:8] - w[0])
