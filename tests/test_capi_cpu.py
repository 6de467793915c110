"""CPU-side checks of the C ABI: the library loads, exports every symbol the
headers declare, and its host-only entry points (lattice bonds, disorder
generators, validation) agree with the oracle / golden vectors.  No compute
call here needs a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='session')
def lib():
    from lsquantumed_gb300.build import build
    build()
    from lsquantumed_gb300 import capi
    return capi.lib()


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, 'include')
    for fn in os.listdir(inc):
        if fn.endswith('.h'):
            src = open(os.path.join(inc, fn)).read()
            src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
            names |= set(re.findall(r'^\s*int\s+(ed_\w+)\s*\(', src, flags=re.M))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 40
    for n in names:
        assert hasattr(lib, n), n


def test_python_signatures_cover_header():
    from lsquantumed_gb300 import capi
    assert set(declared_symbols()) == set(capi.SIGNATURES)


def test_version_and_error_buffer(lib):
    assert lib.ed_version() == 1
    assert lib.ed_last_error(None, 0) >= 0


def _bonds(lib, ltype, n, lx, ly):
    a = np.zeros((4 * n, 2), dtype=np.int32)
    b = np.zeros((4 * n, 2), dtype=np.int32)
    na, nb = ctypes.c_int64(), ctypes.c_int64()
    rc = lib.ed_lattice_bonds(ltype, n, lx, ly, a.ctypes.data, 4 * n, ctypes.byref(na), b.ctypes.data, 4 * n,
                              ctypes.byref(nb))
    return rc, a[:na.value], b[:nb.value]


@pytest.mark.parametrize('case', [(0, 6, 1, 6), (0, 16, 1, 16), (1, 8, 2, 4), (1, 12, 3, 4), (1, 20, 4, 5),
                                  (1, 30, 6, 5), (2, 12, 6, 2), (2, 8, 2, 4), (1, 16, 4, 4)])
def test_lattice_bonds_match_reference_tables(lib, orc, case):
    ltype, n, lx, ly = case
    rc, a, b = _bonds(lib, ltype, n, lx, ly)
    assert rc == 0
    ra, rb = orc.bond_pairs(ltype, n, lx, ly)
    assert np.array_equal(a, ra)
    assert np.array_equal(b, rb)


def test_lattice_rejects_bad_dims(lib):
    rc, _, _ = _bonds(lib, 1, 12, 3, 5)
    assert rc == 1
    rc, _, _ = _bonds(lib, 2, 12, 3, 4)  # honeycomb needs even dims
    assert rc == 1


def test_random_disorder_golden(lib, golden):
    r = golden['random']
    seeds = np.zeros(r['rep'], dtype=np.int64)
    assert lib.ed_random_seeds(1, r['rep'], seeds.ctypes.data) == 0
    assert seeds.tolist() == r['seeds']
    hi = np.zeros(r['nspins'])
    assert lib.ed_random_fields(ctypes.c_int64(int(seeds[r['hi_index']])), r['nspins'], ctypes.c_double(r['min']),
                                ctypes.c_double(r['max']), hi.ctypes.data) == 0
    assert np.allclose(hi, r['hi'], atol=1e-13, rtol=0)


def test_random_generators_match_oracle(lib, orc):
    from lsquantumed_gb300 import ed
    for seed in (0, 1, 17, 511):
        assert np.array_equal(ed.random_fields(seed, 20, -2.0, 2.0), orc.rd_hi(seed, 20, -2.0, 2.0))
        assert np.array_equal(ed.random_normal(seed, 96), orc.normal(seed, 96))


def test_context_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip('GPU present')
    h = ctypes.c_void_p()
    rc = lib.ed_ctx_create(0, None, ctypes.byref(h))
    assert rc != 0
    buf = ctypes.create_string_buffer(512)
    lib.ed_last_error(buf, 512)
    assert buf.value


def test_environment_requires_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip('GPU present')
    import lsquantumed_gb300 as ed
    with pytest.raises(RuntimeError):
        ed.Environment(nspins=8)


def _driver(lib, *args):
    import subprocess
    from lsquantumed_gb300.build import DRIVER
    assert os.path.exists(DRIVER)
    return subprocess.run([DRIVER, *args], capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize('args,msg', [
    (('-n', '7'), 'The total number of spins has to be EVEN.'),
    (('-n', '-4'), 'The total number of spins has to be POSITIVE.'),
    (('-n', '8', '-eps_type', 'lanczos'), 'only -eps_type krylovschur is provided'),
    (('-n',), 'missing value for -n'),
])
def test_driver_rejects_bad_input(lib, args, msg):
    """The drop-in driver validates its flags as the reference's parser and
    Environment do (include/tools/parse_args.hpp:34-66, environment.cpp:31-35)
    before it touches a GPU: exit status 1 and the reference's message."""
    r = _driver(lib, *args)
    assert r.returncode == 1
    assert msg in r.stderr


def test_driver_without_gpu_fails_cleanly(lib):
    """With valid flags and no GPU the driver stops with an error (no CPU
    fallback) and prints no eigenvalue line."""
    import torch
    if torch.cuda.is_available():
        pytest.skip('GPU present')
    r = _driver(lib, '-n', '8', '-ltype', 'chain1D', '-j1', '1', '-d1', '1', '-legacy_unused', '1')
    assert r.returncode == 1
    assert 'warning: unused option -legacy_unused' in r.stderr
    assert 'error: Slepc was not correctly initialized' in r.stderr  # the reference's Environment message
    assert 'CUDA error' in r.stderr and '(ed_capi.cu:' in r.stderr
    assert '||Ax-kx||' not in r.stdout


def test_shim_compiles_for_every_lattice():
    """include/lsqed/lsqed.hpp instantiates with all of the reference's
    interface (Basis, Hamiltonian<L>, Solver::, the four correlations, AF /
    Striped order parameters, DSF_data and DynStructFactor<L, Sqz|Sqp>) for
    every lattice, without warnings."""
    import subprocess
    src = os.path.join(ROOT, 'tests', 'cpp', 'shim_instantiate.cpp')
    r = subprocess.run(['g++', '-std=c++17', '-Wall', '-Wextra', '-Werror', '-fsyntax-only',
                        '-I' + os.path.join(ROOT, 'include'), src], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
