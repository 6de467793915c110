"""ctypes wrapper around the C++ restatement (``liboracle.so``) plus the small
pure-Python pieces of the reference (sublattices, order parameters).

Test infrastructure only; see the package docstring.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, 'ed_oracle.cpp')
_SO = os.path.join(_HERE, 'liboracle.so')
_lock = threading.Lock()
_lib = None

CHAIN1D, SQUARE2D, HONEYCOMB2D = 0, 1, 2
SZSZ, SPSM, SMSP, SISJ = 0, 1, 2, 3


def build(force=False):
    """Compile liboracle.so with g++ (OpenMP).  Idempotent."""
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(_SRC):
        return _SO
    tmp = _SO + '.tmp%d' % os.getpid()
    cmd = ['g++', '-O2', '-std=c++17', '-ffp-contract=off', '-fopenmp', '-fPIC', '-shared', '-o', tmp, _SRC]
    subprocess.check_call(cmd)
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_SO)
            i64, u64, i32, dbl, vp = ctypes.c_int64, ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
            P = ctypes.POINTER
            sig = {
                'orc_compute_size': (i64, [i32, i32]),
                'orc_search_elem': (u64, [i64, i32, i32]),
                'orc_search_index': (i64, [u64, i32]),
                'orc_basis_layout': (i32, [i32, i32, i32, i32, P(i64), P(i64), P(i64)]),
                'orc_generate_basis': (None, [i32, i32, i64, i64, vp]),
                'orc_lattice': (i32, [i32, i32, i32, i32, vp, vp, P(i32), vp, vp, P(i32)]),
                'orc_get_elem_diag': (i64, [i32, i32, i32, i32, i32, u64]),
                'orc_get_coup_elems': (i32, [i32, i32, i32, i32, i32, i32, i32, i32, i64, vp]),
                'orc_get_disorder_elem': (dbl, [u64, i32, vp]),
                'orc_rd_seeds': (None, [i32, i64, vp]),
                'orc_rd_hi': (None, [i64, i32, dbl, dbl, vp]),
                'orc_normal': (None, [i64, i64, vp]),
                'orc_model_create': (vp, [i32, i32, i32, i32, i32, dbl, dbl, dbl, dbl]),
                'orc_model_create_bonds': (vp, [i32, i32, i64, vp, vp, vp]),
                'orc_model_destroy': (None, [vp]),
                'orc_model_dim': (i64, [vp]),
                'orc_model_states': (None, [vp, vp]),
                'orc_set_threads': (None, [i32]),
                'orc_get_threads': (i32, []),
                'orc_model_build': (i64, [vp, i32, vp]),
                'orc_model_csr': (None, [vp, vp, vp, vp]),
                'orc_model_diag': (None, [vp, vp]),
                'orc_model_apply': (None, [vp, vp, vp]),
                'orc_start_vector': (None, [u64, i64, vp]),
                'orc_start_vector_r': (None, [u64, i64, vp]),
                'orc_rows_apply_seeded': (None, [i32, i32, i32, i32, i32, dbl, dbl, dbl, dbl, u64, i32, i64, vp,
                                                 vp]),
                'orc_eps_solve': (i32, [vp, i32, i32, i32, dbl, i32, u64, vp, vp, vp, P(i32), P(i32), P(i64)]),
                'orc_expect': (None, [vp, i32, i32, i32, vp, vp]),
                'orc_sqz': (None, [vp, i32, vp, vp]),
                'orc_sqp': (None, [vp, vp, i32, vp, vp]),
                'orc_vecdot': (None, [i64, vp, vp, vp]),
                'orc_cgs_step': (None, [i64, i32, vp, vp, vp]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


# ---------------------------------------------------------------------------
# Basis / rank (src/basis.cpp, src/hamiltonian.cpp:9-27)
# ---------------------------------------------------------------------------
def compute_size(nspins, nspins_up):
    return lib().orc_compute_size(nspins, nspins_up)


def search_elem(index, nspins, nspins_up):
    return lib().orc_search_elem(index, nspins, nspins_up)


def search_index(state, nspins):
    return lib().orc_search_index(state, nspins)


def basis_layout(nspins, total_mag, mpi_size=1, mpi_rank=0):
    """(size, local_size, global_start_index) or raises ValueError like basis.cpp:66-76."""
    s, l, g = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    rc = lib().orc_basis_layout(nspins, total_mag, mpi_size, mpi_rank, ctypes.byref(s), ctypes.byref(l), ctypes.byref(g))
    if rc:
        raise ValueError('invalid basis (code %d)' % rc)
    return s.value, l.value, g.value


def generate_basis(nspins, nspins_up, start, count):
    out = np.zeros(count, dtype=np.uint64)
    lib().orc_generate_basis(nspins, nspins_up, start, count, _p(out))
    return out


def lattice(ltype, nspins, lx=1, ly=None):
    """Reference neighbour tables: (nn, nnXsite, num_nn, nnn, nnnXsite, num_nnn)."""
    ly = nspins if ly is None else ly
    nn = np.zeros(4 * nspins, dtype=np.int64)
    nnn = np.zeros(4 * nspins, dtype=np.int64)
    nnx = np.zeros(nspins, dtype=np.int64)
    nnnx = np.zeros(nspins, dtype=np.int64)
    a, b = ctypes.c_int(), ctypes.c_int()
    rc = lib().orc_lattice(ltype, nspins, lx, ly, _p(nn), _p(nnx), ctypes.byref(a), _p(nnn), _p(nnnx), ctypes.byref(b))
    if rc:
        raise ValueError('invalid lattice (code %d)' % rc)
    return nn[:(a.value + 1) * nspins], nnx, a.value, nnn[:(b.value + 1) * nspins], nnnx, b.value


def bond_pairs(ltype, nspins, lx=1, ly=None):
    """Flatten the reference tables to ordered (i, j) bond lists for nn and nnn
    (site-major, neighbour order; padding -1 entries skipped via nnXsite)."""
    nn, nnx, a, nnn, nnnx, b = lattice(ltype, nspins, lx, ly)
    out = []
    for tab, cnt, num in ((nn, nnx, a), (nnn, nnnx, b)):
        pairs = []
        for i in range(nspins):
            for k in range(1, cnt[i] + 1):
                pairs.append((i, int(tab[(num + 1) * i + k])))
        out.append(np.array(pairs, dtype=np.int32).reshape(-1, 2))
    return out[0], out[1]


def get_elem_diag(ltype, nspins, lx, ly, nt, state):
    return lib().orc_get_elem_diag(ltype, nspins, lx, ly, nt, state)


def get_coup_elems(ltype, nspins, lx, ly, total_mag, mpi_size, mpi_rank, nt, local_index):
    out = np.zeros(4 * nspins, dtype=np.int64)
    n = lib().orc_get_coup_elems(ltype, nspins, lx, ly, total_mag, mpi_size, mpi_rank, nt, local_index, _p(out))
    if n < 0:
        raise ValueError('bad index')
    return out[:n].tolist()


def get_disorder_elem(state, nspins, hi):
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    return lib().orc_get_disorder_elem(state, nspins, _p(hi))


def rd_seeds(reprod, rep):
    out = np.zeros(rep, dtype=np.int64)
    lib().orc_rd_seeds(1 if reprod else 0, rep, _p(out))
    return out


def rd_hi(seed, nspins, mn, mx):
    out = np.zeros(nspins, dtype=np.float64)
    lib().orc_rd_hi(seed, nspins, mn, mx, _p(out))
    return out


def normal(seed, n):
    out = np.zeros(n, dtype=np.float64)
    lib().orc_normal(seed, n, _p(out))
    return out


def start_vector(seed, n):
    out = np.zeros(n, dtype=np.complex128)
    lib().orc_start_vector(seed, n, _p(out))
    return out


def start_vector_r(seed, n):
    """Real parts of start_vector(seed, n), without the complex copy."""
    out = np.zeros(n, dtype=np.float64)
    lib().orc_start_vector_r(seed, n, _p(out))
    return out


def rows_apply_seeded(ltype, nspins, lx, ly, total_mag, J1, D1, J2, D2, seed, rows, complex_x=False):
    """Rows `rows` of H x for the uniform-coupling Hamiltonian (build_diag +
    build_off_diag), x = start_vector(seed) (its real parts unless complex_x),
    each row evaluated on its own from the reference's per-row rules; no
    basis or matrix is built, so any N whose ranks fit 64 bits works."""
    r = np.ascontiguousarray(rows, dtype=np.int64)
    out = np.zeros(2 * len(r), dtype=np.float64)
    lib().orc_rows_apply_seeded(ltype, nspins, lx, ly, total_mag, J1, D1, J2, D2, seed, 1 if complex_x else 0,
                                len(r), _p(r), _p(out))
    y = out[0::2] + 1j * out[1::2]
    return y if complex_x else y.real.copy()


def vecdot(x, y):
    """PETSc VecDot(x, y) = y^H x."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    y = np.ascontiguousarray(y, dtype=np.complex128)
    out = np.zeros(2)
    lib().orc_vecdot(x.size, _p(x), _p(y), _p(out))
    return complex(out[0], out[1])


def cgs_step(V, w):
    """One CGS pass (h = V^H w; w -= V h) on the CPU; V is (nv, n) complex."""
    h = np.zeros(2 * V.shape[0])
    lib().orc_cgs_step(V.shape[1], V.shape[0], _p(V), _p(w), _p(h))
    return h[0::2] + 1j * h[1::2]


def set_threads(n):
    lib().orc_set_threads(n)


def get_threads():
    return lib().orc_get_threads()


# ---------------------------------------------------------------------------
# Model: basis + lattice + couplings, explicit CSR in the reference layout.
# ---------------------------------------------------------------------------
class Model:
    BUILD_DIAG, BUILD_OFF_DIAG, BUILD_DISORDER = 1, 2, 4

    def __init__(self, ltype, nspins, lx=1, ly=None, total_mag=0, J1=1.0, D1=1.0, J2=0.0, D2=0.0,
                 bonds=None, Jb=None, Db=None):
        ly = nspins if ly is None else ly
        self.nspins, self.total_mag = nspins, total_mag
        self.ltype, self.lx, self.ly = ltype, lx, ly
        if bonds is None:
            self._h = lib().orc_model_create(ltype, nspins, lx, ly, total_mag, J1, D1, J2, D2)
        else:
            pairs = np.ascontiguousarray(bonds, dtype=np.int32)
            Jb = np.ascontiguousarray(Jb, dtype=np.float64)
            Db = np.ascontiguousarray(Db, dtype=np.float64)
            self._h = lib().orc_model_create_bonds(nspins, total_mag, len(pairs), _p(pairs), _p(Jb), _p(Db))
        if not self._h:
            raise ValueError('invalid model')
        self.dim = lib().orc_model_dim(self._h)
        self.nnz = None

    def __del__(self):
        if getattr(self, '_h', None):
            lib().orc_model_destroy(self._h)
            self._h = None

    def states(self):
        out = np.zeros(self.dim, dtype=np.uint64)
        lib().orc_model_states(self._h, _p(out))
        return out

    def build(self, flags=3, hi=None):
        hi_a = None if hi is None else np.ascontiguousarray(hi, dtype=np.float64)
        if hi_a is not None:
            flags |= self.BUILD_DISORDER
        self.nnz = lib().orc_model_build(self._h, flags, None if hi_a is None else _p(hi_a))
        return self.nnz

    def csr(self):
        rp = np.zeros(self.dim + 1, dtype=np.int64)
        cols = np.zeros(self.nnz, dtype=np.int64)
        vals = np.zeros(self.nnz, dtype=np.float64)
        lib().orc_model_csr(self._h, _p(rp), _p(cols), _p(vals))
        return rp, cols, vals

    def scipy(self):
        import scipy.sparse as sp
        rp, cols, vals = self.csr()
        return sp.csr_matrix((vals.astype(np.complex128), cols, rp), shape=(self.dim, self.dim))

    def diag(self):
        out = np.zeros(self.dim, dtype=np.float64)
        lib().orc_model_diag(self._h, _p(out))
        return out

    def apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros_like(x)
        lib().orc_model_apply(self._h, _p(x), _p(y))
        return y

    def eps_solve(self, nev=1, ncv=0, mpd=0, tol=1e-8, max_it=0, seed=0, vectors=True):
        m = max(ncv if ncv > 0 else max(2 * nev, nev + 15), nev)
        m = min(m, self.dim)
        ev = np.zeros(m)
        er = np.zeros(m)
        vec = np.zeros((m, self.dim), dtype=np.complex128) if vectors else None
        nconv, its, nhv = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
        l = lib().orc_eps_solve(self._h, nev, ncv, mpd, tol, max_it, seed, _p(ev), _p(er),
                                None if vec is None else _p(vec),
                                ctypes.byref(nconv), ctypes.byref(its), ctypes.byref(nhv))
        res = {'evals': ev[:l].copy(), 'errs': er[:l].copy(), 'nconv': nconv.value, 'its': its.value,
               'nhv': nhv.value}
        if vec is not None:
            res['evecs'] = vec[:l].copy()
        return res

    def expect(self, op, i, j, psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        out = np.zeros(2)
        lib().orc_expect(self._h, op, i, j, _p(psi), _p(out))
        return complex(out[0], out[1])

    def sqz(self, spin, psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        out = np.zeros_like(psi)
        lib().orc_sqz(self._h, spin, _p(psi), _p(out))
        return out

    def sqp(self, target, spin, psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        out = np.zeros(target.dim, dtype=np.complex128)
        lib().orc_sqp(self._h, target._h, spin, _p(psi), _p(out))
        return out

    def dense(self):
        return self.scipy().toarray()


# ---------------------------------------------------------------------------
# Sublattices (src/sublattice.cpp:5-91) and order parameters
# (include/phys.tmpl_func.hpp:5-81).
# ---------------------------------------------------------------------------
def sublattice_af(ltype, nspins, lx=1, ly=None):
    ly = nspins if ly is None else ly
    sl = [[], []]
    if ltype == CHAIN1D:
        for i in range(nspins):
            sl[1 if i % 2 else 0].append(i)
    else:
        tagx = 0
        for ix in range(lx):
            tagy = tagx
            for iy in range(ly):
                sl[1 if tagy % 2 else 0].append(ix * ly + iy)
                tagy ^= 1
            tagx ^= 1
    return sl


def sublattice_striped(ltype, nspins, lx, ly):
    if ltype != SQUARE2D:
        raise ValueError('striped sublattices are defined for square2D only')
    sl = [[], [], [], []]
    tagx = 0
    for ix in range(lx):
        tagy = 0
        for iy in range(ly):
            cur = ix * ly + iy
            sl[1 if tagy % 2 else 0].append(cur)
            sl[3 if tagx % 2 else 2].append(cur)
            tagy ^= 1
        tagx ^= 1
    return sl


def squared_sublatt_mag_af(model, sublat, psi):
    """phys.tmpl_func.hpp:5-41: 8/(N(N+4)) * sum_l sum_{i,j in l} <S_i.S_j>."""
    e = 0j
    for sl in sublat:
        for i in sl:
            for j in sl:
                e += model.expect(SISJ, i, j, psi)
    n = model.nspins
    return e * 8.0 / n / (n + 4.0)


def squared_sublatt_mag_str(model, sublat, psi):
    """phys.tmpl_func.hpp:45-81: 4/(N(N+4)) * sum over the 4 striped sublattices."""
    e = 0j
    for s in range(2):
        for l in range(2):
            sl = sublat[s * 2 + l]
            for i in sl:
                for j in sl:
                    e += model.expect(SISJ, i, j, psi)
    n = model.nspins
    return e * 4.0 / n / (n + 4.0)


# ---------------------------------------------------------------------------
# S(q, w) post-processing, restated from postprocessing/dynamicStep0_preprocess.ipynb
# (cells 4, 11-13, 15, 17) and the sum-rule check of dynamicStep2_plotSw.ipynb
# (cell 12), in the notebooks' loop order.
# ---------------------------------------------------------------------------
def q_grid(nspins, lx, ly):
    """cell 4: q_i = ((i // Ly) 2 pi / Lx, (i % Ly) 2 pi / Ly), i < nQ = N."""
    pi = np.arccos(-1)
    return np.array([((i // ly) * 2 * pi / lx, (i % ly) * 2 * pi / ly) for i in range(nspins)])


def dsf_spectrum(c, dE, positions, qs, nw=5001, w_min=0.0, w_max=5.0, eps=None):
    """One realisation's S[q][w]: cells 11 (Lorentzian), 12-13 (phase sum,
    |.|^2 / N) and 15 (sum over levels).  c is (N, nev) complex."""
    nspins, nev = c.shape
    eps = 1.0 / nspins if eps is None else eps
    e2 = eps * eps
    inv_pi = 1.0 / np.arccos(-1)
    w = np.linspace(w_min, w_max, nw)
    factor = np.zeros((len(qs), nev))
    for iq, q in enumerate(qs):
        amp = np.zeros(nev, dtype=np.complex128)
        for i in range(nspins):
            amp = amp + np.exp(1j * (q[0] * positions[i][0] + q[1] * positions[i][1])) * c[i, :]
        factor[iq] = np.abs(amp) ** 2 / nspins
    delta = inv_pi * e2 / (e2 + (w[:, None] - np.asarray(dE)[None, :]) ** 2)  # (nw, nev)
    return factor @ delta.T  # (nq, nw)


def dsf_average(spectra):
    """cell 17: 2 pi / rep * sum over realisations."""
    return 2 * np.arccos(-1) * np.sum(spectra, axis=0) / len(spectra)


def dsf_sum_rule(S, w_min=0.0, w_max=5.0):
    """dynamicStep2_plotSw.ipynb cell 12: sum(S) * dw / (2 pi), expected 0.25."""
    dw = (w_max - w_min) / (S.shape[-1] - 1)
    return float(np.sum(S) * dw / (2 * np.arccos(-1)))
