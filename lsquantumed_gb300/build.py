"""Build libedgb300.so (CUDA kernels + C ABI) in-tree for sm_103a.

    python -m lsquantumed_gb300.build        # or lsquantumed_gb300.build.build()

Each translation unit is compiled by nvcc in parallel, then linked into
``lsquantumed_gb300/_lib/libedgb300.so``.  Objects go to ``_build/``.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(ROOT, '_build', 'edgb300')
LIBDIR = os.path.join(HERE, '_lib')
LIB = os.path.join(LIBDIR, 'libedgb300.so')

SOURCES = ['ed_capi.cu', 'ed_basis.cu', 'ed_hamiltonian.cu', 'ed_linalg.cu', 'ed_eps.cu', 'ed_measure.cu',
           'ed_batch.cu', 'ed_adjoint.cu', 'ed_hv_lin.cu',
           'ed_spectrum.cu', 'ed_hv_jit.cu', 'ed_peaks.cu', 'ed_tc.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2', '-Xcompiler', '-fopenmp',
         '--expt-relaxed-constexpr', '-I' + os.path.join(ROOT, 'include')]


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def cuda_lib_dir(cc):
    """The toolkit's library directory next to nvcc (libnvrtc for the
    run-time specialised H.v is loaded from there)."""
    return os.path.normpath(os.path.join(os.path.dirname(os.path.realpath(cc)), '..', 'lib64'))


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.h', '.cuh'))]
    headers.append(os.path.join(ROOT, 'include', 'ed_capi.h'))
    cc = nvcc()
    defs = ['-DED_CUDA_LIB_DIR="%s"' % cuda_lib_dir(cc)]
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace('.cu', '.o'))
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + ARCH + FLAGS + defs + ['-c', s, '-o', o])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, res):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError('nvcc failed: ' + ' '.join(cmd))
    objs = [os.path.join(BUILD, s.replace('.cu', '.o')) for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + '.tmp%d' % os.getpid()
        cmd = [cc] + ARCH + ['-shared', '-o', tmp] + objs + ['-cudart', 'static', '-ldl', '-lgomp']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError('link failed')
        os.replace(tmp, LIB)
    build_driver()
    return LIB


DRIVER_SRC = os.path.join(HERE, 'drivers', 'lsqed_main.cpp')
DRIVER = os.path.join(LIBDIR, 'lsqed_main')


def build_driver():
    """The C++ drop-in driver (lsqed.hpp shim over the C ABI), linked to the library."""
    deps = [DRIVER_SRC, LIB, os.path.join(ROOT, 'include', 'lsqed', 'lsqed.hpp'), os.path.join(ROOT, 'include', 'ed_capi.h')]
    if not _stale(DRIVER, deps):
        return DRIVER
    cmd = ['g++', '-O2', '-std=c++17', '-I' + os.path.join(ROOT, 'include'), DRIVER_SRC, '-o', DRIVER + '.tmp',
           '-L' + LIBDIR, '-ledgb300', '-Wl,-rpath,$ORIGIN']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError('driver build failed')
    os.replace(DRIVER + '.tmp', DRIVER)
    return DRIVER


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
