"""ctypes binding of libedgb300.so (include/ed_capi.h).

The library is built in-tree (``python -m lsquantumed_gb300.build``).  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, '_lib', 'libedgb300.so')

ED_OK, ED_EINVAL, ED_ECUDA, ED_ENOMEM, ED_ESTATE, ED_ENOTCONV, ED_ENOTSUP = range(7)
ED_CHAIN1D, ED_SQUARE2D, ED_HONEYCOMB2D = 0, 1, 2
ED_OP_SZSZ, ED_OP_SPSM, ED_OP_SMSP, ED_OP_SISJ = 0, 1, 2, 3
ED_HAM_MATRIX_FREE, ED_HAM_CSR = 0, 1
ED_ACC_FP64, ED_ACC_EXACT, ED_ACC_FIXED64 = 0, 1, 2
ED_TERM_XY, ED_TERM_ZZ, ED_TERM_Z, ED_TERM_SISJ = 0, 1, 2, 3
ED_RESTART_AUTO, ED_RESTART_FP64, ED_RESTART_PAIR, ED_RESTART_EXACT, ED_RESTART_FIXED = 0, 1, 2, 3, 4

_ERRNAMES = {1: 'EINVAL', 2: 'ECUDA', 3: 'ENOMEM', 4: 'ESTATE', 5: 'ENOTCONV', 6: 'ENOTSUP'}


class EDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__('%s: %s' % (_ERRNAMES.get(code, code), msg))
        self.code = code


class InvalidArgument(EDError, ValueError):
    """Raised where the reference throws std::invalid_argument."""


vp = ctypes.c_void_p
i32 = ctypes.c_int
i64 = ctypes.c_int64
u64 = ctypes.c_uint64
dbl = ctypes.c_double
P = ctypes.POINTER

# name: argtypes (all return int status)
SIGNATURES = {
    'ed_last_error': [ctypes.c_char_p, ctypes.c_size_t],
    'ed_version': [],
    'ed_ctx_create': [i32, vp, P(vp)],
    'ed_ctx_destroy': [vp],
    'ed_ctx_synchronize': [vp],
    'ed_ctx_kernel_count': [vp, P(i64)],
    'ed_ctx_profile': [vp, i32],
    'ed_ctx_profile_read': [vp, P(i64), P(dbl)],
    'ed_probe_rates': [vp, P(dbl), P(dbl), P(dbl)],
    'ed_vec_create': [vp, i64, P(vp)],
    'ed_vec_destroy': [vp],
    'ed_vec_to_host': [vp, vp, vp, i64],
    'ed_vec_from_host': [vp, vp, vp, i64],
    'ed_basis_create': [vp, i32, i32, P(vp)],
    'ed_basis_destroy': [vp],
    'ed_basis_info': [vp, P(i64), P(i32), P(i32), P(i32)],
    'ed_basis_states_host': [vp, i64, i64, vp],
    'ed_basis_rank_host': [vp, vp, vp, i64],
    'ed_basis_unrank_host': [vp, vp, vp, i64],
    'ed_basis_device_states': [vp, P(vp)],
    'ed_lattice_bonds': [i32, i32, i32, i32, vp, i64, P(i64), vp, i64, P(i64)],
    'ed_ham_create': [vp, vp, vp, i64, vp, i64, dbl, dbl, dbl, dbl, P(vp)],
    'ed_ham_create_bonds': [vp, vp, vp, i64, vp, vp, P(vp)],
    'ed_ham_destroy': [vp],
    'ed_ham_build_diag': [vp],
    'ed_ham_build_off_diag': [vp],
    'ed_ham_build_disorder': [vp, vp],
    'ed_ham_apply': [vp, vp, vp],
    'ed_ham_apply_host': [vp, vp, vp],
    'ed_ham_apply_real': [vp, vp, vp],
    'ed_ham_apply_real_dot': [vp, vp, vp, P(dbl), P(dbl)],
    'ed_ham_apply_noalloc': [vp, vp, vp],
    'ed_ham_build_csr': [vp, P(i64)],
    'ed_ham_set_mode': [vp, i32],
    'ed_ham_export_csr_host': [vp, vp, vp, vp, i64],
    'ed_ham_set_accumulation': [vp, i32],
    'ed_ham_diag_host': [vp, vp],
    'ed_ham_size': [vp, P(i64)],
    'ed_ham_hv_variant': [vp, i32, vp, ctypes.c_size_t],
    'ed_ham_set_hv_variant': [vp, ctypes.c_char_p],
    'ed_eps_create': [vp, i32, i32, i32, P(vp)],
    'ed_eps_set_dimensions': [vp, i32, i32, i32],
    'ed_eps_set_tolerances': [vp, dbl, i32],
    'ed_eps_set_seed': [vp, u64],
    'ed_eps_set_restart_arithmetic': [vp, i32],
    'ed_bv_mult_real': [vp, vp, i32, vp, i32, i32, vp, i64, i32],
    'ed_bv_dot_real': [vp, vp, i32, vp, i64, i32, vp],
    'ed_batch_set_restart_arithmetic': [vp, i32],
    'ed_batch_set_hv_tile': [vp, i32, i32],
    'ed_batch_set_graphs': [vp, i32],
    'ed_batch_graph_sweeps': [vp, P(i64)],
    'ed_batch_hv_tile': [vp, P(i32), P(i32)],
    'ed_eps_set_initial_vector': [vp, vp, i32],
    'ed_eps_solve': [vp, P(i32)],
    'ed_eps_get_eigenpair': [vp, i32, P(dbl), P(dbl), vp],
    'ed_eps_get_eigenvector_host': [vp, i32, vp],
    'ed_eps_get_stats': [vp, P(i32), P(i64), P(i32), P(i64)],
    'ed_eps_destroy': [vp],
    'ed_batch_create': [vp, i32, vp, P(vp)],
    'ed_batch_destroy': [vp],
    'ed_batch_apply': [vp, vp, vp],
    'ed_batch_diag_host': [vp, vp],
    'ed_batch_solve': [vp, i32, i32, dbl, i32, u64, vp, vp, vp],
    'ed_batch_solve_many': [vp, i32, i32, i32, dbl, i32, u64, vp, vp, vp],
    'ed_batch_get_eigenvector': [vp, i32, i32, vp],
    'ed_batch_stats': [vp, P(i32), P(i64)],
    'ed_expect_pairs': [vp, i32, vp, vp, i64, vp],
    'ed_expect_all_pairs': [vp, i32, vp, vp],
    'ed_dsf_coefficients': [vp, vp, i32, vp, vp, i32, vp],
    'ed_random_seeds': [i32, i64, vp],
    'ed_random_fields': [i64, i32, dbl, dbl, vp],
    'ed_random_normal': [i64, i64, vp],
    'ed_expect_mixed': [vp, vp, vp, i64, vp, vp, vp],
    'ed_apply_term': [vp, i32, i32, i32, vp, vp],
    'ed_grad_energy': [vp, vp, i64, vp, vp, vp, vp],
    'ed_minres': [vp, dbl, vp, vp, dbl, i32, vp, P(i32), P(dbl)],
    'ed_dsf_spectrum': [vp, i32, i32, vp, vp, i32, vp, vp, i32, dbl, dbl, dbl, vp],
}

_lib = None
_lock = threading.Lock()


def lib():
    """Load libedgb300.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError('libedgb300.so is not built (%s); run python -m lsquantumed_gb300.build'
                                   % LIB_PATH)
            L = ctypes.CDLL(LIB_PATH)
            for name, args in SIGNATURES.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = ctypes.c_int
            _lib = L
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().ed_last_error(buf, 1024)
    return buf.value.decode(errors='replace')


def check(rc):
    if rc != ED_OK:
        msg = last_error()
        if rc == ED_EINVAL:
            raise InvalidArgument(rc, msg)
        raise EDError(rc, msg)
    return rc


def call(name, *args):
    return check(getattr(lib(), name)(*args))
