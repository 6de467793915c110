"""The reference's own drivers compile against the C++ shim.

Each of examples/main.cpp, main_disorder.cpp, main_NO_disorder.cpp and
ex1-4.cpp from the reference tree is copied with every #include line
replaced by `#include <lsqed/lsqed_dropin.hpp>`, compiled with g++ and
linked against libedgb300.so; nothing else in the source changes.  (Running
them needs a GPU; tests/test_gpu_driver.py runs the shim's own driver.)
The reference tree is read from $LSQUANTUMED_REF (the variable
tests/golden/make_golden.py reads); the test is skipped when it is absent.
"""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get('LSQUANTUMED_REF', '')
DRIVERS = ['main.cpp', 'main_disorder.cpp', 'main_NO_disorder.cpp', 'ex1.cpp', 'ex2.cpp', 'ex3.cpp', 'ex4.cpp']


@pytest.fixture(scope='module')
def libdir():
    from lsquantumed_gb300.build import build
    build()
    return os.path.join(ROOT, 'lsquantumed_gb300', '_lib')


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, 'examples')), reason='LSQUANTUMED_REF not set')
@pytest.mark.parametrize('name', DRIVERS)
def test_reference_driver_compiles(libdir, tmp_path, name):
    src = open(os.path.join(REF, 'examples', name)).read()
    lines = src.split('\n')
    out, replaced = [], False
    for line in lines:
        if re.match(r'\s*#\s*include\b', line):
            if not replaced:
                out.append('#include <lsqed/lsqed_dropin.hpp>')
                replaced = True
            continue
        out.append(line)
    body_ref = [l for l in lines if not re.match(r'\s*#\s*include\b', l)]
    body_new = [l for l in out if l != '#include <lsqed/lsqed_dropin.hpp>']
    assert body_ref == body_new  # only the #include lines differ
    f = tmp_path / name
    f.write_text('\n'.join(out))
    exe = tmp_path / (name[:-4] + '.x')
    r = subprocess.run(['g++', '-std=c++17', '-O1', '-I' + os.path.join(ROOT, 'include'), str(f), '-o', str(exe),
                        '-L' + libdir, '-ledgb300', '-Wl,-rpath,' + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert exe.exists()
