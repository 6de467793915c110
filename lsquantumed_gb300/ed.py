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
    def dsf_weights(c, positions, q):
        """|sum_i e^{i q.r_i} c_{i,n}|^2 / N for each level n (the weight the
        post-processing notebooks form from the dsf files)."""
        ph = np.exp(1j * (positions @ np.asarray(q, dtype=np.float64)))
        amp = ph @ c
        return np.abs(amp) ** 2 / c.shape[0]
