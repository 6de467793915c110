"""Host-side mirror of LSQuantumED's hot-path interfaces over the C ABI.

Class and method names follow the reference so a caller of
``Basis`` / ``Hamiltonian<L>`` / ``Solver::`` / ``SiSj`` / ``Phys::`` finds the
same entry points (file:line citations are relative to the LSQuantumED tree).
Device vectors are ``torch.complex128`` CUDA tensors; torch is used only for
device memory.  All compute runs in libedgb300.so.
"""
import ctypes
import math
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import capi
from .capi import InvalidArgument, call

PETSC_DEFAULT = -2
PETSC_DECIDE = -1


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError('lsquantumed_gb300 needs a CUDA GPU; none is available')
    return torch


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else ctypes.c_void_p(a.data_ptr())


def as_device_vector(x, n=None):
    """Return a contiguous complex128 CUDA tensor holding x."""
    torch = _torch()
    if isinstance(x, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.complex128)).cuda()
    else:
        t = x.to(device='cuda', dtype=torch.complex128).contiguous()
    if n is not None and t.numel() != n:
        raise InvalidArgument(capi.ED_EINVAL, 'vector length %d != basis size %d' % (t.numel(), n))
    return t


def restart_code(mode):
    m = {'auto': capi.ED_RESTART_AUTO, 'fp64': capi.ED_RESTART_FP64, 'pair': capi.ED_RESTART_PAIR,
         'exact': capi.ED_RESTART_EXACT, 'fixed': capi.ED_RESTART_FIXED}.get(mode)
    if m is None:
        raise InvalidArgument(capi.ED_EINVAL, 'unknown restart arithmetic %r' % (mode,))
    return m


def bv_mult_real(env, V, Y, out=None, arith='auto'):
    """out[:, c] = sum_i V[:, i] Y[i, c] for real device vectors: the
    Krylov-Schur restart combination on its own (ed_bv_mult_real).  V is a
    list of m float64 CUDA tensors of n entries, Y an (m, l) array; returns
    the l output tensors."""
    torch = _torch()
    m = len(V)
    Yh = np.ascontiguousarray(Y, dtype=np.float64)
    if Yh.ndim != 2 or Yh.shape[0] != m:
        raise InvalidArgument(capi.ED_EINVAL, 'Y must be (m, l)')
    n = V[0].numel()
    l = Yh.shape[1]
    for v in V:
        if v.dtype != torch.float64 or v.numel() != n or not v.is_cuda or not v.is_contiguous():
            raise InvalidArgument(capi.ED_EINVAL, 'V must hold contiguous float64 CUDA vectors of one length')
    if out is None:
        out = [torch.empty(n, dtype=torch.float64, device=V[0].device) for _ in range(l)]
    vp = (ctypes.c_void_p * m)(*[v.data_ptr() for v in V])
    op = (ctypes.c_void_p * l)(*[o.data_ptr() for o in out])
    call('ed_bv_mult_real', env.handle, vp, m, _p(Yh), l, l, op, n, restart_code(arith))
    return out


def bv_dot_real(env, V, w, arith='auto'):
    """h[i] = V[i]^T w for real device vectors (ed_bv_dot_real): the
    Gram-Schmidt projection on its own.  V: list of float64 CUDA tensors with
    entries of magnitude <= 1, w: float64 CUDA tensor; returns numpy h."""
    torch = _torch()
    m = len(V)
    n = w.numel()
    for v in list(V) + [w]:
        if v.dtype != torch.float64 or v.numel() != n or not v.is_cuda or not v.is_contiguous():
            raise InvalidArgument(capi.ED_EINVAL, 'V and w must be contiguous float64 CUDA vectors of one length')
    h = np.zeros(m)
    vp = (ctypes.c_void_p * m)(*[v.data_ptr() for v in V])
    call('ed_bv_dot_real', env.handle, vp, m, _p(w), n, restart_code(arith), _p(h))
    return h


# ---------------------------------------------------------------------------
# Environment (src/environment.cpp:8-49)
# ---------------------------------------------------------------------------
class Environment:
    """Holds the GPU context; ``nspins`` and ``disorder_flg`` as in the reference.

    There is one process per GPU, so ``mpi_size`` is 1 and ``mpi_rank`` 0."""

    def __init__(self, argv=None, nspins=0, device=0, help=''):
        if nspins:
            if nspins % 2 != 0:
                raise InvalidArgument(capi.ED_EINVAL, 'The total number of spins has to be EVEN.')
            if nspins <= 0:
                raise InvalidArgument(capi.ED_EINVAL, 'The total number of spins has to be POSITIVE.')
        _torch()
        self.nspins = nspins
        self.mpi_rank = 0
        self.mpi_size = 1
        self.disorder_flg = False
        self.device = device
        torch = _torch()
        # Bind the context to torch's current stream so library work is
        # ordered with torch's copies; the legacy default stream (handle 0)
        # is passed as cudaStreamLegacy (1).
        with torch.cuda.device(device):
            sh = torch.cuda.current_stream().cuda_stream
        h = ctypes.c_void_p()
        call('ed_ctx_create', device, ctypes.c_void_p(sh if sh else 1), ctypes.byref(h))
        self._h = h

    @property
    def handle(self):
        return self._h

    def synchronize(self):
        call('ed_ctx_synchronize', self._h)

    def kernel_count(self):
        c = ctypes.c_int64()
        call('ed_ctx_kernel_count', self._h, ctypes.byref(c))
        return c.value

    def profile(self, enable=True):
        """Start (clearing) or stop CUDA-event timing of the H.v launches."""
        call('ed_ctx_profile', self._h, 1 if enable else 0)

    def probe_rates(self):
        """Measured TFLOP/s of FP64 FMA, FP64 tensor mma and FP16/FP32 tensor mma
        on this device (ed_probe_rates)."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        call('ed_probe_rates', self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return {'dfma_tflops': a.value, 'dmma_f64_tflops': b.value, 'hmma_f16_f32_tflops': c.value}

    def profile_read(self):
        """(H.v launches, summed device milliseconds) since profile(True)."""
        n, ms = ctypes.c_int64(), ctypes.c_double()
        call('ed_ctx_profile_read', self._h, ctypes.byref(n), ctypes.byref(ms))
        return n.value, ms.value

    def close(self):
        if getattr(self, '_h', None):
            capi.lib().ed_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Basis (src/basis.cpp:56-94, include/basis.hpp:67-93)
# ---------------------------------------------------------------------------
class Basis:
    def __init__(self, env: Environment, total_mag: int):
        self.env = env
        h = ctypes.c_void_p()
        call('ed_basis_create', env.handle, env.nspins, total_mag, ctypes.byref(h))
        self._h = h
        size, ns, nup, tm = ctypes.c_int64(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call('ed_basis_info', h, ctypes.byref(size), ctypes.byref(ns), ctypes.byref(nup), ctypes.byref(tm))
        self.nspins = ns.value
        self.max_mag = self.nspins // 2
        self.total_mag = tm.value
        self.nspins_up = nup.value
        self.size = size.value
        self.mpi_size = 1
        self.mpi_rank = 0
        self.local_size = self.size
        self.global_start_index = 0
        self._int_basis = None

    @property
    def handle(self):
        return self._h

    @property
    def int_basis(self):
        """The basis states in ascending order (basis.cpp:192-215), numpy uint64."""
        if self._int_basis is None:
            out = np.zeros(self.size, dtype=np.uint64)
            call('ed_basis_states_host', self._h, 0, self.size, _p(out))
            self._int_basis = out
        return self._int_basis

    def search_index(self, states):
        """HamiltHelper::search_index (src/hamiltonian.cpp:9-27) for many states."""
        s = np.ascontiguousarray(np.atleast_1d(states), dtype=np.uint64)
        r = np.zeros(s.size, dtype=np.int64)
        call('ed_basis_rank_host', self._h, _p(s), _p(r), s.size)
        return r

    def search_elem(self, index):
        """BasisHelper::search_elem (src/basis.cpp:9-36) for many indices."""
        r = np.ascontiguousarray(np.atleast_1d(index), dtype=np.int64)
        s = np.zeros(r.size, dtype=np.uint64)
        call('ed_basis_unrank_host', self._h, _p(r), _p(s), r.size)
        return s

    def __del__(self):
        if getattr(self, '_h', None):
            try:
                capi.lib().ed_basis_destroy(self._h)
            except Exception:
                pass
            self._h = None


# ---------------------------------------------------------------------------
# Lattices (src/lattice.cpp, include/lattice.hpp:166-329)
# ---------------------------------------------------------------------------
class Lattice:
    ltype = None

    def __init__(self, env, nx=1, ny=None):
        self.nspins = env.nspins
        self.nspins_x = nx
        self.nspins_y = env.nspins if ny is None else ny
        cap = 4 * self.nspins
        a = np.zeros((cap, 2), dtype=np.int32)
        b = np.zeros((cap, 2), dtype=np.int32)
        na, nb = ctypes.c_int64(), ctypes.c_int64()
        call('ed_lattice_bonds', self.ltype, self.nspins, self.nspins_x, self.nspins_y, _p(a), cap,
             ctypes.byref(na), _p(b), cap, ctypes.byref(nb))
        self.nn_pairs = a[:na.value].copy()
        self.nnn_pairs = b[:nb.value].copy()

    def num_spins(self):
        return self.nspins

    def get_type(self):
        return self.ltype


class chain1D(Lattice):
    ltype = capi.ED_CHAIN1D

    def __init__(self, env):
        super().__init__(env, 1, env.nspins)

    def num_nn(self):
        return 1

    def num_nnn(self):
        return 1


class square2D(Lattice):
    ltype = capi.ED_SQUARE2D

    def num_nn(self):
        return 2

    def num_nnn(self):
        return 2


class honeycomb2D(Lattice):
    ltype = capi.ED_HONEYCOMB2D

    def num_nn(self):
        return 2

    def num_nnn(self):
        return 3


# ---------------------------------------------------------------------------
# Hamiltonian (include/hamiltonian.hpp:187-299, hamiltonian.tmpl_func.hpp)
# ---------------------------------------------------------------------------
class Hamiltonian:
    def __init__(self, env, basis: Basis, lattice: Optional[Lattice], J1=1.0, Delta1=1.0, J2=0.0, Delta2=0.0,
                 bonds=None, Jb=None, Db=None):
        self.env = env
        self.basis = basis
        self.lattice = lattice
        self.J1, self.Delta1, self.J2, self.Delta2 = J1, Delta1, J2, Delta2
        self.size = basis.size
        h = ctypes.c_void_p()
        if bonds is None:
            nn = np.ascontiguousarray(lattice.nn_pairs, dtype=np.int32)
            nnn = np.ascontiguousarray(lattice.nnn_pairs, dtype=np.int32)
            call('ed_ham_create', env.handle, basis.handle, _p(nn), len(nn), _p(nnn), len(nnn),
                 float(J1), float(Delta1), float(J2), float(Delta2), ctypes.byref(h))
        else:
            pairs = np.ascontiguousarray(bonds, dtype=np.int32).reshape(-1, 2)
            Jb = np.ascontiguousarray(Jb, dtype=np.float64)
            Db = np.ascontiguousarray(Db, dtype=np.float64)
            call('ed_ham_create_bonds', env.handle, basis.handle, _p(pairs), len(pairs), _p(Jb), _p(Db),
                 ctypes.byref(h))
        self._h = h

    @property
    def hamilt(self):
        """The reference exposes ``Mat hamilt``; here the operator itself."""
        return self

    @classmethod
    def from_bonds(cls, env, basis, pairs, J, D):
        """Per-bond couplings J_b, D_b (generalisation; no counterpart in the reference)."""
        return cls(env, basis, None, bonds=pairs, Jb=J, Db=D)

    @property
    def handle(self):
        return self._h

    def build_diag(self, env=None):
        call('ed_ham_build_diag', self._h)
        return 0

    def build_off_diag(self, env=None):
        call('ed_ham_build_off_diag', self._h)
        return 0

    def build_disorder(self, env, hi):
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        if hi.size < self.basis.nspins:
            raise InvalidArgument(capi.ED_EINVAL, 'hi needs nspins entries')
        call('ed_ham_build_disorder', self._h, _p(hi))
        if env is not None:
            env.disorder_flg = True
        return 0

    def hamilt_size(self):
        return self.size

    def hamilt_J1(self):
        return self.J1

    def hamilt_J2(self):
        return self.J2

    def hamilt_D1(self):
        return self.Delta1

    def hamilt_D2(self):
        return self.Delta2

    def apply(self, x, out=None):
        """y = H x (MatMult).  x: CUDA tensor or numpy array; returns a CUDA tensor."""
        torch = _torch()
        xd = as_device_vector(x, self.size)
        y = out if out is not None else torch.empty_like(xd)
        call('ed_ham_apply', self._h, _p(xd), _p(y))
        return y

    def apply_real(self, x, out=None):
        """y = H x for a real vector (float64 CUDA tensor or numpy array) in real
        storage: the real part of apply(x + 0j), bit for bit, at half the
        traffic.  Needs the matrix-free 'fixed64' H.v with uniform couplings."""
        torch = _torch()
        if isinstance(x, np.ndarray):
            x = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64))
        if x.dtype != torch.float64 or x.numel() != self.size:
            raise InvalidArgument(capi.ED_EINVAL, 'expected a float64 vector of %d entries' % self.size)
        xd = x.to('cuda').contiguous()
        y = out if out is not None else torch.empty_like(xd)
        if y.dtype != torch.float64 or y.numel() != self.size or not y.is_contiguous():
            raise InvalidArgument(capi.ED_EINVAL, 'out must be a contiguous float64 vector of %d entries' % self.size)
        call('ed_ham_apply_real', self._h, _p(xd), _p(y))
        return y

    def apply_real_dot(self, x, out=None):
        """(y, x^T y, ||y||^2) with y = H x in real storage, the three formed in
        one pass over the rows (the product the eigensolver runs).  y equals
        apply_real(x) bit for bit."""
        torch = _torch()
        if isinstance(x, np.ndarray):
            x = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64))
        if x.dtype != torch.float64 or x.numel() != self.size:
            raise InvalidArgument(capi.ED_EINVAL, 'expected a float64 vector of %d entries' % self.size)
        xd = x.to('cuda').contiguous()
        y = out if out is not None else torch.empty_like(xd)
        if y.dtype != torch.float64 or y.numel() != self.size or not y.is_contiguous():
            raise InvalidArgument(capi.ED_EINVAL, 'out must be a contiguous float64 vector of %d entries' % self.size)
        xy, yy = ctypes.c_double(), ctypes.c_double()
        call('ed_ham_apply_real_dot', self._h, _p(xd), _p(y), ctypes.byref(xy), ctypes.byref(yy))
        return y, xy.value, yy.value

    def mult(self, x, y):
        call('ed_ham_apply', self._h, _p(x), _p(y))
        return 0

    def apply_host(self, x):
        """y = H x with host (numpy) buffers: copies in and out inside the call."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        call('ed_ham_apply_host', self._h, _p(x), _p(y))
        return y

    def build_csr(self):
        nnz = ctypes.c_int64()
        call('ed_ham_build_csr', self._h, ctypes.byref(nnz))
        return nnz.value

    def set_mode(self, mode):
        call('ed_ham_set_mode', self._h, capi.ED_HAM_CSR if mode in ('csr', capi.ED_HAM_CSR) else
             capi.ED_HAM_MATRIX_FREE)

    def set_accumulation(self, kind):
        """Matrix-free H.v accumulation: 'exact' (128-bit integer sums of block
        floating point input, default), 'fixed64' (64-bit fixed point input) or
        'fp64'."""
        k = {'exact': capi.ED_ACC_EXACT, 'fixed64': capi.ED_ACC_FIXED64, 'fp64': capi.ED_ACC_FP64}[kind]
        call('ed_ham_set_accumulation', self._h, k)

    def set_hv_variant(self, name):
        """Force the matrix-free H.v launch variant ('auto' = autotuner)."""
        call('ed_ham_set_hv_variant', self._h, name.encode())

    def hv_variant(self, dot=False):
        """Launch variant of the matrix-free H.v chosen by the autotuner."""
        buf = ctypes.create_string_buffer(64)
        call('ed_ham_hv_variant', self._h, 1 if dot else 0, buf, 64)
        return buf.value.decode()

    def export_csr(self):
        """(rowptr, cols, vals) of the assembled matrix, rows sorted by column."""
        nnz = self.build_csr()
        rp = np.zeros(self.size + 1, dtype=np.int64)
        cols = np.zeros(max(nnz, 1), dtype=np.int64)
        vals = np.zeros(max(nnz, 1), dtype=np.float64)
        call('ed_ham_export_csr_host', self._h, _p(rp), _p(cols), _p(vals), nnz)
        return rp, cols[:nnz], vals[:nnz]

    def diagonal(self):
        out = np.zeros(self.size, dtype=np.float64)
        call('ed_ham_diag_host', self._h, _p(out))
        return out

    def __del__(self):
        if getattr(self, '_h', None):
            try:
                capi.lib().ed_ham_destroy(self._h)
            except Exception:
                pass
            self._h = None


# ---------------------------------------------------------------------------
# Solver (src/solver.cpp:7-68)
# ---------------------------------------------------------------------------
class EPS:
    def __init__(self, hamilt: Hamiltonian, nev, ncv, mpd):
        self.hamilt = hamilt
        h = ctypes.c_void_p()
        call('ed_eps_create', hamilt.handle, int(nev), int(ncv), int(mpd), ctypes.byref(h))
        self._h = h
        self.nev = nev

    @property
    def handle(self):
        return self._h

    def set_dimensions(self, nev, ncv=PETSC_DEFAULT, mpd=PETSC_DEFAULT):
        call('ed_eps_set_dimensions', self._h, int(nev), int(ncv), int(mpd))
        self.nev = nev

    def set_tolerances(self, tol=0.0, max_it=0):
        call('ed_eps_set_tolerances', self._h, float(tol), int(max_it))

    def set_seed(self, seed):
        call('ed_eps_set_seed', self._h, int(seed))

    def set_restart_arithmetic(self, mode):
        """Products of the restart combination V Y in a real-storage solve:
        'fp64', 'pair' (float pairs on the FP32 units, storage and sums FP64;
        below FP64 accuracy), 'exact' (exact slices on the tensor cores for
        the restart and the Gram-Schmidt projections, ncv <= 32), 'fixed'
        (the restart on the integer units: 56-bit fixed point per row and
        column, exact products, one rounding) or 'auto'."""
        call('ed_eps_set_restart_arithmetic', self._h, restart_code(mode))

    def set_initial_vector(self, v):
        """EPSSetInitialSpace with one vector: numpy (host) or CUDA tensor."""
        if v is None:
            call('ed_eps_set_initial_vector', self._h, None, 0)
        elif isinstance(v, np.ndarray):
            v = np.ascontiguousarray(v, dtype=np.complex128)
            call('ed_eps_set_initial_vector', self._h, _p(v), 0)
        else:
            if v.numel() != self.hamilt.size or not v.is_contiguous():
                raise InvalidArgument(capi.ED_EINVAL, 'initial vector must be contiguous with basis size entries')
            call('ed_eps_set_initial_vector', self._h, _p(v), 1 if v.is_cuda else 0)

    def stats(self):
        its, nhv, nrep, op = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_int64()
        call('ed_eps_get_stats', self._h, ctypes.byref(its), ctypes.byref(nhv), ctypes.byref(nrep), ctypes.byref(op))
        return {'its': its.value, 'nhv': nhv.value, 'nreported': nrep.value, 'ortho_passes': op.value}

    def destroy(self):
        if getattr(self, '_h', None):
            capi.lib().ed_eps_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Solver:
    """Namespace Solver:: (src/solver.cpp).  -eps_* options are applied through
    ``options`` (the reference's EPSSetFromOptions, solver.cpp:21)."""

    options = {}

    @staticmethod
    def SolverInit(matrix: Hamiltonian, nev, ncv=PETSC_DEFAULT, mpd=PETSC_DEFAULT):
        eps = EPS(matrix, nev, ncv, mpd)
        o = Solver.options
        if 'eps_nev' in o or 'eps_ncv' in o or 'eps_mpd' in o:
            eps.set_dimensions(o.get('eps_nev', nev), o.get('eps_ncv', ncv), o.get('eps_mpd', mpd))
        eps.set_tolerances(o.get('eps_tol', 0.0), o.get('eps_max_it', 0))
        return eps

    @staticmethod
    def EPSSetDimensions(eps: EPS, nev, ncv=PETSC_DEFAULT, mpd=PETSC_DEFAULT):
        eps.set_dimensions(nev, ncv, mpd)
        return 0

    @staticmethod
    def EPSSetTolerances(eps: EPS, tol, max_it=0):
        eps.set_tolerances(tol, max_it)
        return 0

    @staticmethod
    def solve(env, eps: EPS):
        n = ctypes.c_int()
        call('ed_eps_solve', eps.handle, ctypes.byref(n))
        return n.value

    @staticmethod
    def solution(eps: EPS, index, vec=None):
        """(eigenvalue, eigenvector CUDA tensor, relative error)."""
        torch = _torch()
        e, err = ctypes.c_double(), ctypes.c_double()
        if vec is None:
            vec = torch.empty(eps.hamilt.size, dtype=torch.complex128, device='cuda')
        call('ed_eps_get_eigenpair', eps.handle, int(index), ctypes.byref(e), ctypes.byref(err), _p(vec))
        return e.value, vec, err.value

    @staticmethod
    def eigenvalue(eps: EPS, index):
        e, err = ctypes.c_double(), ctypes.c_double()
        call('ed_eps_get_eigenpair', eps.handle, int(index), ctypes.byref(e), ctypes.byref(err), None)
        return e.value, err.value

    @staticmethod
    def solution_host(eps: EPS, index, out=None):
        """Eigenvector into host memory (numpy, or a pinned torch CPU tensor)."""
        v = np.zeros(eps.hamilt.size, dtype=np.complex128) if out is None else out
        call('ed_eps_get_eigenvector_host', eps.handle, int(index), _p(v))
        return v

    @staticmethod
    def SolverClean(eps: EPS):
        eps.destroy()
        return 0


# ---------------------------------------------------------------------------
# Batched disorder sweep (the loop of examples/main_disorder.cpp:82-120)
# ---------------------------------------------------------------------------
class DisorderBatch:
    """B field realisations of one Hamiltonian, solved together.

    ``fields`` is (B, N): realisation b uses h_i = fields[b, i] exactly as
    build_disorder would.  Vectors are (dim, B) CUDA tensors."""

    def __init__(self, hamilt: Hamiltonian, fields):
        f = np.ascontiguousarray(fields, dtype=np.float64)
        if f.ndim != 2 or f.shape[1] != hamilt.basis.nspins:
            raise InvalidArgument(capi.ED_EINVAL, 'fields must be (B, nspins)')
        self.hamilt = hamilt
        self.B = f.shape[0]
        h = ctypes.c_void_p()
        call('ed_batch_create', hamilt.handle, self.B, _p(f), ctypes.byref(h))
        self._h = h

    def apply(self, X, out=None):
        torch = _torch()
        X = X.to(device='cuda', dtype=torch.complex128).contiguous()
        Y = torch.empty_like(X) if out is None else out
        call('ed_batch_apply', self._h, _p(X), _p(Y))
        return Y

    def diagonal(self):
        out = np.zeros((self.hamilt.size, self.B), dtype=np.float64)
        call('ed_batch_diag_host', self._h, _p(out))
        return out

    def set_restart_arithmetic(self, mode):
        """Products of the restart combination: 'fp64', 'pair' or 'auto'
        (FP64; pairs only on request)."""
        if mode == 'exact':
            raise InvalidArgument(capi.ED_EINVAL, "the batched sweep has no 'exact' restart")
        call('ed_batch_set_restart_arithmetic', self._h, restart_code(mode))

    def set_hv_tile(self, rows, threads):
        """Force the batched H.v tile: rows per CTA tile (4, 8, 16, 32) and
        threads per CTA (128, 256); (0, 0) re-enables the autotuner."""
        call('ed_batch_set_hv_tile', self._h, int(rows), int(threads))

    def set_graphs(self, on=True):
        """Capture every expansion sweep after the first in a CUDA graph
        (ed_batch_set_graphs; on by default, False launches directly)."""
        call('ed_batch_set_graphs', self._h, 1 if on else 0)

    def graph_sweeps(self):
        """Sweeps of the last solve that ran from a CUDA graph."""
        n = ctypes.c_int64()
        call('ed_batch_graph_sweeps', self._h, ctypes.byref(n))
        return n.value

    def hv_tile(self):
        """(rows, threads) of the batched H.v tile in use; (0, 0) before the
        autotuner has run."""
        r, t = ctypes.c_int32(), ctypes.c_int32()
        call('ed_batch_hv_tile', self._h, ctypes.byref(r), ctypes.byref(t))
        return r.value, t.value

    def solve(self, nev=1, ncv=0, tol=1e-8, max_it=0, seed=0):
        ev = np.zeros((self.B, nev))
        er = np.zeros((self.B, nev))
        nc = np.zeros(self.B, dtype=np.int32)
        call('ed_batch_solve', self._h, int(nev), int(ncv), float(tol), int(max_it), int(seed), _p(ev), _p(er),
             _p(nc))
        its, nhv = ctypes.c_int(), ctypes.c_int64()
        call('ed_batch_stats', self._h, ctypes.byref(its), ctypes.byref(nhv))
        return {'evals': ev, 'errs': er, 'nconv': nc, 'its': its.value, 'nhv': nhv.value}

    def eigenvector(self, b, i):
        torch = _torch()
        v = torch.empty(self.hamilt.size, dtype=torch.complex128, device='cuda')
        call('ed_batch_get_eigenvector', self._h, int(b), int(i), _p(v))
        return v

    def __del__(self):
        if getattr(self, '_h', None):
            try:
                capi.lib().ed_batch_destroy(self._h)
            except Exception:
                pass
            self._h = None


def solve_batches(batches, nev=1, ncv=0, tol=1e-8, max_it=0, seed=0):
    """Solve several DisorderBatch objects at once (ed_batch_solve_many): each
    on its own host thread and stream, so the device overlaps them.  Every
    batch must come from a different Environment.  Returns one result dict
    per batch, as DisorderBatch.solve."""
    k = len(batches)
    evs = [np.zeros((bt.B, nev)) for bt in batches]
    ers = [np.zeros((bt.B, nev)) for bt in batches]
    ncs = [np.zeros(bt.B, dtype=np.int32) for bt in batches]
    hp = (ctypes.c_void_p * k)(*[bt._h for bt in batches])
    ep = (ctypes.c_void_p * k)(*[a.ctypes.data for a in evs])
    rp = (ctypes.c_void_p * k)(*[a.ctypes.data for a in ers])
    np_ = (ctypes.c_void_p * k)(*[a.ctypes.data for a in ncs])
    call('ed_batch_solve_many', hp, k, int(nev), int(ncv), float(tol), int(max_it), int(seed), ep, rp, np_)
    out = []
    for bt, ev, er, nc in zip(batches, evs, ers, ncs):
        its, nhv = ctypes.c_int(), ctypes.c_int64()
        call('ed_batch_stats', bt._h, ctypes.byref(its), ctypes.byref(nhv))
        out.append({'evals': ev, 'errs': er, 'nconv': nc, 'its': its.value, 'nhv': nhv.value})
    return out


# ---------------------------------------------------------------------------
# Correlations (src/spinOperators/correlation.cpp)
# ---------------------------------------------------------------------------
class Correlation:
    op = None

    def __init__(self, env, basis: Basis):
        self.env = env
        self.basis = basis

    def ExpectVal(self, env, spin_i, spin_j, state):
        return self.ExpectValPairs([(spin_i, spin_j)], state)[0]

    def ExpectValPairs(self, pairs, state):
        psi = as_device_vector(state, self.basis.size)
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        out = np.zeros(len(pr), dtype=np.complex128)
        call('ed_expect_pairs', self.basis.handle, self.op, _p(psi), _p(pr), len(pr), _p(out))
        return out

    def AllPairs(self, state):
        psi = as_device_vector(state, self.basis.size)
        n = self.basis.nspins
        out = np.zeros(n * n, dtype=np.complex128)
        call('ed_expect_all_pairs', self.basis.handle, self.op, _p(psi), _p(out))
        return out.reshape(n, n)


class SzSz(Correlation):
    op = capi.ED_OP_SZSZ


class SpSm(Correlation):
    op = capi.ED_OP_SPSM


class SmSp(Correlation):
    op = capi.ED_OP_SMSP


class SiSj(Correlation):
    op = capi.ED_OP_SISJ


# ---------------------------------------------------------------------------
# Sublattices (src/sublattice.cpp:5-91)
# ---------------------------------------------------------------------------
class AF:
    def __init__(self, lattice: Lattice, size=2):
        n, lx, ly = lattice.nspins, lattice.nspins_x, lattice.nspins_y
        self.sublat = [[], []]
        if isinstance(lattice, chain1D):
            for i in range(n):
                self.sublat[1 if i % 2 else 0].append(i)
        else:
            tagx = 0
            for ix in range(lx):
                tagy = tagx
                for iy in range(ly):
                    self.sublat[1 if tagy % 2 else 0].append(ix * ly + iy)
                    tagy ^= 1
                tagx ^= 1

    def get_size(self):
        return 2

    def get_sl(self, i):
        return self.sublat[i]


class Striped:
    def __init__(self, lattice: Lattice, size=4):
        if not isinstance(lattice, square2D):
            raise InvalidArgument(capi.ED_EINVAL, 'striped sublattices are defined for square2D')
        lx, ly = lattice.nspins_x, lattice.nspins_y
        self.sublat = [[], [], [], []]
        tagx = 0
        for ix in range(lx):
            tagy = 0
            for iy in range(ly):
                cur = ix * ly + iy
                self.sublat[1 if tagy % 2 else 0].append(cur)
                self.sublat[3 if tagx % 2 else 2].append(cur)
                tagy ^= 1
            tagx ^= 1

    def get_size(self):
        return 4

    def get_sl(self, i):
        return self.sublat[i]


# ---------------------------------------------------------------------------
# Disorder (src/tools/random_disorder.cpp)
# ---------------------------------------------------------------------------
class RandomDisorder:
    def __init__(self, nspins, reprod=True, min=-0.3, max=0.3, rep=1):
        self.nspins, self.min, self.max, self.rep = nspins, min, max, rep
        self.srand_seq = np.zeros(rep, dtype=np.int64)
        call('ed_random_seeds', 1 if reprod else 0, rep, _p(self.srand_seq))
        self.hi = np.zeros(nspins, dtype=np.float64)

    def hi_init(self, dis_index):
        call('ed_random_fields', int(self.srand_seq[dis_index]), self.nspins, float(self.min), float(self.max),
             _p(self.hi))
        return self.hi


def random_fields(seed, nspins, lo, hi):
    out = np.zeros(nspins, dtype=np.float64)
    call('ed_random_fields', int(seed), nspins, float(lo), float(hi), _p(out))
    return out


def random_normal(seed, n):
    out = np.zeros(n, dtype=np.float64)
    call('ed_random_normal', int(seed), int(n), _p(out))
    return out


# ---------------------------------------------------------------------------
# Phys (include/phys.hpp, include/phys.tmpl_func.hpp)
# ---------------------------------------------------------------------------
@dataclass
class DSF_data:
    b0: Basis = None
    b1: Basis = None
    lat: Lattice = None
    h0: Hamiltonian = None
    h1: Hamiltonian = None
    nev: int = 10
    ncv: int = PETSC_DECIDE
    mpd: int = PETSC_DECIDE
    disorder: bool = False
    hi: Optional[np.ndarray] = None
    path: str = './'


class Phys:
    @staticmethod
    def _sum_sublattice_pairs(env, basis, lists, state):
        pairs = [(i, j) for sl in lists for i in sl for j in sl]
        vals = SiSj(env, basis).ExpectValPairs(pairs, state)
        return vals.sum()

    @staticmethod
    def SquaredSubLattMagAF(env, basis, sublat: AF, state):
        """8/(N(N+4)) sum_l sum_{i,j in l} <S_i.S_j> (phys.tmpl_func.hpp:5-41)."""
        e = Phys._sum_sublattice_pairs(env, basis, [sublat.get_sl(l) for l in range(sublat.get_size())], state)
        n = env.nspins
        return e * 8.0 / n / (n + 4.0)

    @staticmethod
    def SquaredSubLattMagSTR(env, basis, sublat: Striped, state):
        """4/(N(N+4)) sum over the striped sublattices (phys.tmpl_func.hpp:45-81)."""
        e = Phys._sum_sublattice_pairs(env, basis, [sublat.get_sl(s * 2 + l) for s in range(2) for l in range(2)],
                                       state)
        n = env.nspins
        return e * 4.0 / n / (n + 4.0)

    @staticmethod
    def dsf_coefficients(env, b0, b1, op, psi0, vecs):
        """c[i, n] = <v_n| S_i |psi0> for all sites; vecs is (nev, dim1) on the device."""
        torch = _torch()
        psi = as_device_vector(psi0, b0.size)
        V = vecs.to(device='cuda', dtype=torch.complex128).contiguous()
        nev = V.shape[0]
        c = np.zeros((b0.nspins, nev), dtype=np.complex128)
        call('ed_dsf_coefficients', b0.handle, b1.handle, int(op), _p(psi), _p(V), nev, _p(c))
        return c

    @staticmethod
    def DynStructFactor(env, data: DSF_data, gs, state, dis_iter=0, SQ='Sqz', write=True):
        """Phys::DynStructFactor (phys.tmpl_func.hpp:87-215): eigensolve of h1 for
        nev pairs, coefficients c_{i,n} = VecDot(SQ_i |state>, v_n), and the
        ``dsf_d<k>.dat`` file in the reference format.  Returns (E_n - gs, c)."""
        torch = _torch()
        eps = Solver.SolverInit(data.h1, data.nev, data.ncv, data.mpd)
        nconv = Solver.solve(env, eps)
        if nconv < data.nev:
            raise RuntimeError('DSF eigensolve converged %d < nev=%d pairs' % (nconv, data.nev))
        vecs = torch.empty((data.nev, data.h1.size), dtype=torch.complex128, device='cuda')
        evals = []
        for n in range(data.nev):
            e, _, _ = Solver.solution(eps, n, vecs[n])
            evals.append(e)
        op = 0 if SQ == 'Sqz' else 1
        c = Phys.dsf_coefficients(env, data.b0, data.b1, op, state, vecs)
        Solver.SolverClean(eps)
        dE = np.array(evals) - float(np.real(gs))
        if write:
            Phys.write_dsf_file(env, data, gs, dis_iter, dE, c)
        return dE, c

    @staticmethod
    def write_dsf_file(env, data: DSF_data, gs, dis_iter, dE, c):
        """Byte layout of phys.tmpl_func.hpp:126-200."""
        path = os.path.join(data.path, 'dsf_d%d.dat' % dis_iter)
        h0 = data.h0
        with open(path, 'w') as f:
            f.write('#------------------------------- Parameters -------------------------------------\n')
            f.write('#%7s:   %d  \n' % (' nspins', env.nspins))
            f.write('#%7s:   %d  \n' % (' nev', data.nev))
            f.write('#%7s:   %.16f  \n' % (' GS', float(np.real(gs))))
            f.write('#%7s:   %.5f  %4s:   %.5f  %4s:   %.5f  %4s:   %.5f\n' %
                    ('J1', h0.hamilt_J1(), 'D1', h0.hamilt_D1(), 'J2', h0.hamilt_J2(), 'D2', h0.hamilt_D2()))
            if data.disorder:
                for i in range(env.nspins):
                    f.write('# hi[%4d]: %.16f\n' % (i, data.hi[i]))
            f.write('#--------------------------------------------------------------------------------\n#\n#\n')
            f.write('#----- Energy -----  ------ Factor -----\n')
            for spin in range(env.nspins):
                f.write('# spin: %d\n' % spin)
                for n in range(data.nev):
                    f.write('%.13e  %.13e\n' % (dE[n], c[spin, n].real))
        return path

    @staticmethod
    def site_positions(lattice: Lattice):
        """r_i = (i // ly, i % ly) for square2D, (0, i) for chain1D."""
        n, ly = lattice.nspins, lattice.nspins_y
        return np.array([(i // ly, i % ly) for i in range(n)], dtype=np.float64)

    @staticmethod
    def q_grid(lattice: Lattice):
        """The notebooks' wave vectors (dynamicStep0_preprocess.ipynb cell 4):
        q_i = ((i // ly) 2 pi / lx, (i % ly) 2 pi / ly), i < N."""
        n, lx, ly = lattice.nspins, lattice.nspins_x, lattice.nspins_y
        return np.array([((i // ly) * 2 * np.pi / lx, (i % ly) * 2 * np.pi / ly) for i in range(n)])

    @staticmethod
    def dsf_spectrum(env, c, dE, positions, qs, nw=5001, w_min=0.0, w_max=5.0, eps=None, out=None):
        """S(q, w) on the device from DSF coefficients c (N x nev) and level
        energies dE (nev): Lorentzian-broadened weights as in the
        post-processing notebook (dynamicStep0_preprocess.ipynb cells 11-15),
        eps = 1/N by default.  Accumulates into `out` (a (nq, nw) float64
        CUDA tensor) when given, so realisations sum; returns the tensor."""
        torch = _torch()
        c = np.ascontiguousarray(c, dtype=np.complex128)
        nspins, nev = c.shape
        dE = np.ascontiguousarray(dE, dtype=np.float64)
        qs = np.ascontiguousarray(np.asarray(qs, dtype=np.float64).reshape(-1, 2))
        r = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).reshape(-1, 2))
        if dE.size != nev or r.shape[0] != nspins:
            raise InvalidArgument(capi.ED_EINVAL, 'c must be (N, nev), dE (nev), positions (N, 2)')
        if eps is None:
            eps = 1.0 / nspins
        S = out if out is not None else torch.zeros((len(qs), nw), dtype=torch.float64, device='cuda')
        call('ed_dsf_spectrum', env.handle, nspins, nev, _p(c), _p(dE), len(qs), _p(qs), _p(r), int(nw),
             float(w_min), float(w_max), float(eps), _p(S))
        return S

    @staticmethod
    def dsf_sum_rule(S, w_min=0.0, w_max=5.0):
        """sum_{q,w} S dw / (2 pi) of a disorder-averaged S(q, w) (already
        scaled by 2 pi / rep), the notebooks' check against 1/4
        (dynamicStep2_plotSw.ipynb cell 12)."""
        S = S.cpu().numpy() if hasattr(S, 'cpu') else np.asarray(S)
        dw = (w_max - w_min) / (S.shape[-1] - 1)
        return float(S.sum() * dw / (2 * np.pi))

    @staticmethod
    def dsf_weights(c, positions, q):
        """|sum_i e^{i q.r_i} c_{i,n}|^2 / N for each level n (the weight the
        post-processing notebooks form from the dsf files)."""
        ph = np.exp(1j * (positions @ np.asarray(q, dtype=np.float64)))
        amp = ph @ c
        return np.abs(amp) ** 2 / c.shape[0]


# ---------------------------------------------------------------------------
# Adjoint gradients (no counterpart in the reference: its couplings are
# uniform and it forms no derivatives).
#   H = sum_b [J_b XY_b + D_b ZZ_b] + sum_i h_i S^z_i,
#   XY_b = (S+_i S-_j + S-_i S+_j)/2,  ZZ_b = S^z_i S^z_j.
# ---------------------------------------------------------------------------
class Adjoint:
    """Hellmann-Feynman energy gradients and adjoint (MINRES) gradients of
    ground-state expectation values with respect to J_b, D_b and h_i."""
    XY, ZZ, Z, SISJ = capi.ED_TERM_XY, capi.ED_TERM_ZZ, capi.ED_TERM_Z, capi.ED_TERM_SISJ

    @staticmethod
    def _terms(terms):
        t = np.asarray(terms, dtype=np.int64).reshape(-1, 3)
        kinds = np.ascontiguousarray(t[:, 0], dtype=np.int32)
        ij = np.ascontiguousarray(t[:, 1:], dtype=np.int32)
        return kinds, ij

    @staticmethod
    def expect_mixed(basis: Basis, terms, lam, psi):
        """<lam| O_t |psi> for terms (kind, i, j); complex array."""
        lam = as_device_vector(lam, basis.size)
        psi = as_device_vector(psi, basis.size)
        kinds, ij = Adjoint._terms(terms)
        out = np.zeros(len(kinds), dtype=np.complex128)
        call('ed_expect_mixed', basis.handle, _p(kinds), _p(ij), len(kinds), _p(lam), _p(psi), _p(out))
        return out

    @staticmethod
    def apply_term(basis: Basis, kind, i, j, psi, out=None):
        torch = _torch()
        psi = as_device_vector(psi, basis.size)
        y = torch.empty_like(psi) if out is None else out
        call('ed_apply_term', basis.handle, int(kind), int(i), int(j), _p(psi), _p(y))
        return y

    @staticmethod
    def energy_gradient(basis: Basis, pairs, psi):
        """(dE/dJ_b, dE/dD_b, dE/dh_i) at the eigenvector psi (Hellmann-Feynman;
        valid for a non-degenerate level)."""
        psi = as_device_vector(psi, basis.size)
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        dJ = np.zeros(len(pr))
        dD = np.zeros(len(pr))
        dh = np.zeros(basis.nspins)
        call('ed_grad_energy', basis.handle, _p(pr), len(pr), _p(psi), _p(dJ), _p(dD), _p(dh))
        return dJ, dD, dh

    @staticmethod
    def eigenvalue_sum_gradient(eps, pairs, k):
        """Gradient of E_0 + ... + E_{k-1} (the lowest k levels of a solved
        EPS) with respect to (J_b, D_b, h_i): the sum of the levels'
        Hellmann-Feynman expectations.  Valid when level k-1 is not part of a
        multiplet that continues past k (a trace over whole multiplets does
        not depend on the basis chosen inside them)."""
        basis = eps.hamilt.basis
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        gJ = np.zeros(len(pr))
        gD = np.zeros(len(pr))
        gh = np.zeros(basis.nspins)
        for n in range(int(k)):
            _, v, _ = Solver.solution(eps, n)
            dJ, dD, dh = Adjoint.energy_gradient(basis, pr, v)
            gJ += dJ
            gD += dD
            gh += dh
        return gJ, gD, gh

    @staticmethod
    def minres(hamilt: Hamiltonian, shift, rhs, q=None, tol=1e-12, max_it=0):
        """x with (H - shift) x = rhs on the complement of the unit vector q."""
        torch = _torch()
        b = as_device_vector(rhs, hamilt.size)
        qd = None if q is None else as_device_vector(q, hamilt.size)
        x = torch.empty_like(b)
        its, rel = ctypes.c_int(), ctypes.c_double()
        call('ed_minres', hamilt.handle, float(shift), _p(b), None if qd is None else _p(qd), float(tol),
             int(max_it), _p(x), ctypes.byref(its), ctypes.byref(rel))
        return x, its.value, rel.value

    @staticmethod
    def apply_observable(basis: Basis, observable, psi):
        """O psi for O = sum_t c_t O_t, observable = [(c, kind, i, j), ...]."""
        torch = _torch()
        psi = as_device_vector(psi, basis.size)
        acc = torch.zeros_like(psi)
        tmp = torch.empty_like(psi)
        for c, kind, i, j in observable:
            Adjoint.apply_term(basis, kind, i, j, psi, out=tmp)
            acc.add_(tmp, alpha=complex(c))
        return acc

    @staticmethod
    def expectation_gradient(hamilt: Hamiltonian, pairs, e0, psi0, observable, tol=1e-12, max_it=0):
        """Gradient of <psi0|O|psi0> (psi0 the normalised, non-degenerate ground
        state, e0 its energy) with respect to (J_b, D_b, h_i):
        (H - e0) lam = P (O psi0), P = 1 - psi0 psi0^H, then
        d<O>/dtheta = -2 Re <lam| dH/dtheta |psi0>.
        Returns (value, dJ, dD, dh, info)."""
        basis = hamilt.basis
        psi = as_device_vector(psi0, basis.size)
        nrm = float(np.sqrt(np.real(psi.conj().dot(psi).item())))
        psi = psi / nrm
        opsi = Adjoint.apply_observable(basis, observable, psi)
        val = psi.conj().dot(opsi).item()
        rhs = opsi - val * psi
        lam, its, rel = Adjoint.minres(hamilt, e0, rhs, q=psi, tol=tol, max_it=max_it)
        pr = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        terms = [(Adjoint.XY, i, j) for i, j in pr] + [(Adjoint.ZZ, i, j) for i, j in pr] + \
                [(Adjoint.Z, i, i) for i in range(basis.nspins)]
        g = -2.0 * np.real(Adjoint.expect_mixed(basis, terms, lam, psi))
        nb = len(pr)
        return float(np.real(val)), g[:nb], g[nb:2 * nb], g[2 * nb:], {'its': its, 'relres': rel}


def ground_state_energy(env, basis: Basis, pairs, J, D, h=None, nev=1, ncv=0, tol=1e-12):
    """E0(J, D, h) as a differentiable torch function of per-bond couplings
    (J, D: float64 tensors of len(pairs)) and site fields h (len nspins, or
    None).  The backward pass is the Hellmann-Feynman gradient."""
    torch = _torch()
    pairs_np = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))

    class _E0(torch.autograd.Function):
        @staticmethod
        def forward(ctx, J, D, hf):
            ham = Hamiltonian.from_bonds(env, basis, pairs_np, J.detach().cpu().numpy(), D.detach().cpu().numpy())
            ham.build_diag(env)
            ham.build_off_diag(env)
            if hf is not None and hf.numel():
                ham.build_disorder(env, hf.detach().cpu().numpy())
            eps = Solver.SolverInit(ham, nev, ncv if ncv else PETSC_DEFAULT)
            Solver.EPSSetTolerances(eps, tol)
            Solver.solve(env, eps)
            e0, _ = Solver.eigenvalue(eps, 0)
            v = torch.empty(basis.size, dtype=torch.complex128, device='cuda')
            Solver.solution(eps, 0, v)
            dJ, dD, dh = Adjoint.energy_gradient(basis, pairs_np, v)
            Solver.SolverClean(eps)
            ctx.has_h = hf is not None and hf.numel() > 0
            ctx.save_for_backward(torch.from_numpy(dJ).to(J.device), torch.from_numpy(dD).to(D.device),
                                  torch.from_numpy(dh).to(hf.device))
            return torch.tensor(float(e0), dtype=torch.float64, device=J.device)

        @staticmethod
        def backward(ctx, g):
            dJ, dD, dh = ctx.saved_tensors
            return g * dJ, g * dD, (g * dh if ctx.has_h else None)

    hf = h if h is not None else torch.zeros(0, dtype=torch.float64)
    return _E0.apply(J, D, hf)
