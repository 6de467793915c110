/*
 * ed_capi.h — C ABI of the GB300 exact-diagonalization engine (libedgb300.so).
 *
 * The engine replaces LSQuantumED's hot path (fixed-Sz basis -> Hamiltonian
 * application -> Krylov-Schur eigensolve -> correlations / DSF) on one GPU.
 * Every entry point names the reference interface it replaces (paths are
 * relative to the LSQuantumED source tree).
 *
 * Conventions
 *  - Return value: ED_OK (0) or an ED_E* code; ed_last_error() gives the
 *    message of the most recent failure on the calling thread.
 *  - Pointers whose name ends in _dev are device pointers on the context's
 *    device; _host pointers are host memory.  Vectors are complex128,
 *    interleaved (re, im), length = basis size, in basis (rank) order.
 *  - States are bit strings (bit i set = site i up), exactly as
 *    Basis::int_basis (include/basis.hpp:67-75).
 *  - All work is issued on the context's stream; calls returning host data
 *    synchronize that stream.
 */
#ifndef ED_CAPI_H
#define ED_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ED_OK = 0,
  ED_EINVAL = 1,    /* bad argument (std::invalid_argument in the reference) */
  ED_ECUDA = 2,     /* CUDA runtime error */
  ED_ENOMEM = 3,    /* device allocation failed */
  ED_ESTATE = 4,    /* call out of order (e.g. eigenpair before solve) */
  ED_ENOTCONV = 5,  /* solver hit max_it before nev pairs converged */
  ED_ENOTSUP = 6    /* size outside what the device path supports */
};

enum { ED_CHAIN1D = 0, ED_SQUARE2D = 1, ED_HONEYCOMB2D = 2 };  /* lattice_type, include/lattice.hpp */
enum { ED_OP_SZSZ = 0, ED_OP_SPSM = 1, ED_OP_SMSP = 2, ED_OP_SISJ = 3 };  /* spinOperators/correlation.hpp */
enum { ED_HAM_MATRIX_FREE = 0, ED_HAM_CSR = 1 };
enum { ED_ACC_FP64 = 0, ED_ACC_EXACT = 1, ED_ACC_FIXED64 = 2 };

typedef struct { double re, im; } ed_cplx;
typedef struct ed_ctx ed_ctx;
typedef struct ed_basis ed_basis;
typedef struct ed_ham ed_ham;
typedef struct ed_eps ed_eps;

/* ---- errors / version ---------------------------------------------------- */
int ed_last_error(char* buf, size_t len);
int ed_version(void);

/* ---- context: replaces Environment (src/environment.cpp:8-49) ------------- */
/* device < 0 selects the current device.  stream may be NULL (the context
 * creates its own non-blocking stream) or a cudaStream_t owned by the caller. */
int ed_ctx_create(int device, void* stream, ed_ctx** out);
int ed_ctx_destroy(ed_ctx* ctx);
int ed_ctx_synchronize(ed_ctx* ctx);
/* Number of kernels this context launched so far (for launch accounting). */
int ed_ctx_kernel_count(const ed_ctx* ctx, int64_t* count);
/* Per-launch timing of the H.v kernels with CUDA events on the context's
 * stream (the reference's -log_view / TIME_CODE timers,
 * include/tools/time_monitor.hpp:45-112).  enable != 0 clears and starts. */
int ed_ctx_profile(ed_ctx* ctx, int enable);
/* H.v launches recorded and their summed device time in milliseconds. */
int ed_ctx_profile_read(ed_ctx* ctx, int64_t* n_hv, double* ms_hv);

/* Arithmetic rates of the units the dense contractions could use, measured on
 * the context's device in TFLOP/s (register-resident loops on every SM, CUDA
 * events): FP64 FMA, FP64 tensor mma (m8n8k4), and FP16-input FP32-accumulate
 * tensor mma (m16n8k16).  Any output may be NULL.  No counterpart in the
 * reference; for the benchmark's reports. */
int ed_probe_rates(ed_ctx* ctx, double* dfma_tflops, double* dmma_tflops, double* hmma_tflops);

/* ---- device vectors: replace MatCreateVecs / VecDestroy / VecGetArray ---- */
/* n complex128 entries on the context's device (uninitialised). */
int ed_vec_create(ed_ctx* ctx, int64_t n, ed_cplx** vec_dev);
int ed_vec_destroy(ed_cplx* vec_dev);
/* Copies on the context's stream; the host side returns after completion. */
int ed_vec_to_host(ed_ctx* ctx, const ed_cplx* vec_dev, ed_cplx* host, int64_t n);
int ed_vec_from_host(ed_ctx* ctx, const ed_cplx* host, ed_cplx* vec_dev, int64_t n);

/* ---- basis: replaces Basis(env, total_mag) (src/basis.cpp:56-94) ---------- */
/* Validates like basis.cpp:66-76 (|total_mag| <= N/2; N even, > 0 like
 * environment.cpp:31-35); N <= 32 on the device path (ED_ENOTSUP otherwise). */
int ed_basis_create(ed_ctx* ctx, int nspins, int total_mag, ed_basis** out);
int ed_basis_destroy(ed_basis* b);
/* size = C(N, nspins_up) (basis.cpp:38-46). */
int ed_basis_info(const ed_basis* b, int64_t* size, int* nspins, int* nspins_up, int* total_mag);
/* int_basis[start .. start+count) (basis.cpp:192-215) into host memory. */
int ed_basis_states_host(const ed_basis* b, int64_t start, int64_t count, uint64_t* out_host);
/* Rank of each state: HamiltHelper::search_index (src/hamiltonian.cpp:9-27). */
int ed_basis_rank_host(const ed_basis* b, const uint64_t* states_host, int64_t* ranks_host, int64_t n);
/* Unrank: BasisHelper::search_elem (src/basis.cpp:9-36). */
int ed_basis_unrank_host(const ed_basis* b, const int64_t* ranks_host, uint64_t* states_host, int64_t n);
/* Device array of the basis states (uint32 words, one per state). */
int ed_basis_device_states(const ed_basis* b, const uint32_t** states_dev);

/* ---- lattice: replaces chain1D / square2D / honeycomb2D (src/lattice.cpp) -- */
/* Flattened ordered bond lists (i, j) for nn and nnn, in the order
 * get_coup_elems / get_elem_diag visit them (site-major, neighbour order;
 * hamiltonian.tmpl_func.hpp:350-426).  Capacities in pairs; n_* receive the
 * counts.  Returns ED_EINVAL on lx*ly != N (lattice.cpp:67-68). */
int ed_lattice_bonds(int ltype, int nspins, int lx, int ly,
                     int32_t* nn_pairs, int64_t nn_cap, int64_t* n_nn,
                     int32_t* nnn_pairs, int64_t nnn_cap, int64_t* n_nnn);

/* ---- Hamiltonian: replaces Hamiltonian<L> (include/hamiltonian.hpp:187-249) */
/* Hamiltonian<L>(env, basis, lattice, J1, Delta1, J2, Delta2)
 * (hamiltonian.tmpl_func.hpp:70-91): nn and nnn bond lists plus couplings. */
int ed_ham_create(ed_ctx* ctx, const ed_basis* b,
                  const int32_t* nn_pairs, int64_t n_nn, const int32_t* nnn_pairs, int64_t n_nnn,
                  double J1, double D1, double J2, double D2, ed_ham** out);
/* Generalisation with one (J_b, D_b) per bond (per-bond couplings; the
 * reference has only the uniform J1/J2).  Diagonal = sum_b D_b*0.25*(+-1). */
int ed_ham_create_bonds(ed_ctx* ctx, const ed_basis* b, const int32_t* pairs, int64_t nbonds,
                        const double* J_host, const double* D_host, ed_ham** out);
int ed_ham_destroy(ed_ham* h);
/* build_diag (hamiltonian.tmpl_func.hpp:129-225). */
int ed_ham_build_diag(ed_ham* h);
/* build_off_diag (hamiltonian.tmpl_func.hpp:229-344): enables the J terms. */
int ed_ham_build_off_diag(ed_ham* h);
/* build_disorder (hamiltonian.tmpl_func.hpp:97-125): the diagonal becomes
 * D1*0.25*E_nn + D2*0.25*E_nnn + 0.5*sum_i(+-h_i).  hi has N entries. */
int ed_ham_build_disorder(ed_ham* h, const double* hi_host);
/* y = H x (PETSc MatMult on Hamiltonian::hamilt).  Device vectors. */
int ed_ham_apply(ed_ham* h, const ed_cplx* x_dev, ed_cplx* y_dev);
/* Same with host buffers (copies in and out on the context's stream). */
int ed_ham_apply_host(ed_ham* h, const ed_cplx* x_host, ed_cplx* y_host);
/* y = H x for real vectors (double[dim] on the device).  The Hamiltonian is
 * real symmetric, so this is ed_ham_apply on x + 0i with half the storage and
 * traffic; the result equals the real part of ed_ham_apply's bit for bit.
 * Needs the matrix-free two-table kernel (ED_ACC_FIXED64; for per-bond
 * couplings, the run-time compiled form): ED_ENOTSUP otherwise.  No counterpart in the reference (PETSc vectors there
 * are complex128). */
int ed_ham_apply_real(ed_ham* h, const double* x_dev, double* y_dev);
/* ed_ham_apply_real fused with the two reductions a Lanczos step takes from
 * the product: *xy_host = x^T y and *yy_host = ||y||^2 (either may be NULL),
 * in the same pass over the rows (the H.v the eigensolver runs).  y equals
 * ed_ham_apply_real's bit for bit.  Synchronises the context's stream.  No
 * counterpart in the reference (SLEPc forms these with separate VecDot /
 * VecNorm calls after MatMult). */
int ed_ham_apply_real_dot(ed_ham* h, const double* x_dev, double* y_dev, double* xy_host, double* yy_host);
/* y = H x (device vectors) without allocating any device memory: for
 * callers that cannot let a library call cudaMalloc, e.g. code running under
 * a framework that owns the whole device memory pool, or a loop that cannot
 * afford the synchronisation an allocation may bring.  No counterpart in the
 * reference.  Same fixed-point H.v as ed_ham_apply (ED_ACC_FIXED64), with its
 * scratch in one static device array reserved when the library's module is
 * loaded, so every GPU that loads the library holds ED_NOALLOC_MAX_STATES *
 * 16 + 256 bytes (64 MiB) until the process exits.  Limits: at most
 * ED_NOALLOC_MAX_STATES basis states (ED_EINVAL beyond), uniform J1/J2
 * Hamiltonians only (ED_ENOTSUP for per-bond ones).  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture.  The address belongs to the
 * device's context: after a device reset (cudaDeviceReset, or a framework
 * resetting the primary context) the next call sees a new current context
 * and looks the address up again, so make that call, too, outside a stream
 * capture.  All calls share the array: calls that overlap on the GPU race on
 * it, so order them. */
#define ED_NOALLOC_MAX_STATES (1 << 22)
int ed_ham_apply_noalloc(ed_ham* h, const ed_cplx* x_dev, ed_cplx* y_dev);
/* Explicit CSR on the device (when it fits); then ed_ham_set_mode(ED_HAM_CSR)
 * makes ed_ham_apply / the solver use the CSR SpMV. */
int ed_ham_build_csr(ed_ham* h, int64_t* nnz);
int ed_ham_set_mode(ed_ham* h, int mode);
/* Export the assembled matrix (rows sorted by column, duplicates summed in
 * the reference's order) — the parity view of Hamiltonian::hamilt. */
int ed_ham_export_csr_host(ed_ham* h, int64_t* rowptr_host, int64_t* cols_host, double* vals_host, int64_t cap);
/* Matrix-free H.v accumulation (no counterpart in the reference, whose PETSc
 * MatMult adds in FP64):
 *   ED_ACC_EXACT (default): the input is kept as block floating point (62-bit
 *     mantissas, one exponent per 32 states) and the gathered entries are
 *     summed exactly in 128-bit integers, then rounded once to FP64;
 *   ED_ACC_FIXED64: the input is quantised to 64-bit fixed point against its
 *     largest entry (error <= 2^-57 of max|x| per entry), sums exact in
 *     int64, rounded once to FP64;
 *   ED_ACC_FP64: gathered entries added in FP64.
 * Per-bond Hamiltonians (ed_ham_create_bonds) with ED_ACC_FIXED64 use the
 * run-time compiled two-table kernel where NVRTC is available: each bond's
 * J_b / 2 becomes a 64-bit fixed-point constant (relative error below 2^-60
 * of the largest coupling), each row's sum of c_b * xq is exact in 128 bits
 * and rounded once; elsewhere, and with the other modes, they add in FP64. */
int ed_ham_set_accumulation(ed_ham* h, int kind);
/* Diagonal of the assembled matrix (MatGetDiagonal). */
int ed_ham_diag_host(ed_ham* h, double* out_host);
int ed_ham_size(const ed_ham* h, int64_t* size);
/* Name of the matrix-free H.v launch variant the autotuner chose (dot = 0:
 * plain H.v, 1: H.v fused with x^H y), "" before the first H.v or when the
 * operator does not use the two-table kernel.  No counterpart in the
 * reference; for reports. */
int ed_ham_hv_variant(const ed_ham* h, int dot, char* buf, size_t len);
/* Force the matrix-free H.v launch variant: "u4-b6", "u4-b4", "u8-b4",
 * "u8-b1" (static kernels: unroll depth and register budget), "jit" /
 * "jit-b4" / "jit-b3" (kernel compiled at run time for this operator's bonds,
 * blocks of 256 threads, 2 / 4 / 3 blocks per SM), "jit-w3" / "jit-w4" (the
 * same with one block of 768 / 1024 threads per SM) or "auto" (autotuner,
 * the default).  All variants give bit-identical results.  ED_ENOTSUP for
 * operators that do not use the two-table kernel (CSR, FP64 or 128-bit
 * accumulation), and for a static variant on a per-bond operator (only the
 * run-time compiled ones exist there).  No counterpart in the reference. */
int ed_ham_set_hv_variant(ed_ham* h, const char* name);

/* ---- eigensolver: replaces Solver:: (src/solver.cpp:7-68) ----------------- */
/* SolverInit(eps, H, nev, ncv, mpd): Hermitian, Krylov-Schur, smallest real.
 * ncv/mpd <= 0 mean PETSC_DECIDE (ncv = max(2 nev, nev + 15), capped at n).
 * The solver refers to h until ed_eps_destroy: destroy it first (as an EPS
 * is cleaned before the Mat it solves in the reference's drivers); the same
 * holds for a batch (ed_batch_destroy before ed_ham_destroy). */
int ed_eps_create(ed_ham* h, int nev, int ncv, int mpd, ed_eps** out);
/* EPSSetDimensions */
int ed_eps_set_dimensions(ed_eps* e, int nev, int ncv, int mpd);
/* -eps_tol / -eps_max_it (tol <= 0: 1e-8, max_it <= 0: max(100, 2n/ncv)). */
int ed_eps_set_tolerances(ed_eps* e, double tol, int max_it);
/* Seed of the deterministic start vector (re, im ~ U[-1,1) per entry). */
int ed_eps_set_seed(ed_eps* e, uint64_t seed);
/* Arithmetic of the restart combination V Y (the Krylov-Schur restart;
 * BVMultInPlace in SLEPc) in a real-storage solve (a real start vector and
 * the two-table H.v).  ED_RESTART_FP64: FP64 FMA beside exact integer
 * products.  ED_RESTART_PAIR: float-pair products on the FP32 units (each
 * FP64 value split into hi + lo, error below 2^-45 of |v y| per product;
 * storage and sums stay FP64), below FP64 accuracy, so only on request.
 * ED_RESTART_EXACT: exact slices on the tensor cores for the restart
 * combination and the Gram-Schmidt projections (ed_bv_mult_real,
 * ed_bv_dot_real; ncv <= 32).  ED_RESTART_FIXED: the restart combination on
 * the integer units: each row of V in 56-bit fixed point against the row's
 * largest entry, each column of Y against its own, exact products of 28-bit
 * limbs, one rounding per output (error below 2^-51 of max|V row| * max|Y
 * column|; ncv <= 32, FP64 beyond).  ED_RESTART_AUTO (default):
 * ED_RESTART_FP64.  No counterpart in the reference (FP64 throughout). */
#define ED_RESTART_AUTO 0
#define ED_RESTART_FP64 1
#define ED_RESTART_PAIR 2
#define ED_RESTART_EXACT 3
#define ED_RESTART_FIXED 4
int ed_eps_set_restart_arithmetic(ed_eps* e, int mode);
/* The restart combination on its own: out_c = sum_{i<m} V_i Y[i*ldY + c] for
 * c < l, real device vectors of n entries (V_dev and out_dev: host arrays of
 * device pointers; out must not alias V; Y on the host).  This is SLEPc's
 * BVMultInPlace inside the Krylov-Schur restart (reached from EPSSolve,
 * src/solver.cpp:45).  arith: ED_RESTART_FP64, ED_RESTART_PAIR, or
 * ED_RESTART_EXACT: the products on the tensor cores in exact 8-bit slices of
 * 63-bit fixed point (per 128-row tile of V, per column of Y), level sums
 * combined exactly and rounded once to FP64 (m <= 32, ED_ENOTSUP beyond);
 * ED_RESTART_FIXED: 56-bit fixed point per row of V and column of Y, exact
 * integer products (m <= 32; the FP64 form beyond); ED_RESTART_AUTO picks
 * what the solver would by default.
 * Synchronises the stream. */
int ed_bv_mult_real(ed_ctx* ctx, const double* const* V_dev, int m, const double* Y_host, int ldY, int l,
                    double* const* out_dev, int64_t n, int arith);
/* The Gram-Schmidt projection on its own: h_host[i] = V_i^T w, i < m, real
 * device vectors of n entries with |V_i entries| <= 1 (orthonormal columns,
 * as in the Krylov basis); SLEPc's BVDotVec in the orthogonalisation of the
 * Krylov-Schur expansion (reached from EPSSolve, src/solver.cpp:45).
 * arith: ED_RESTART_FP64 / ED_RESTART_AUTO (FP64 FMA), or ED_RESTART_EXACT:
 * the products on the tensor cores in exact 8-bit slices of 63-bit fixed
 * point (per 128-row tile and column), summed exactly within each CTA,
 * rounded once per slice level and CTA and summed in FP64 across CTAs.
 * Synchronises the stream. */
int ed_bv_dot_real(ed_ctx* ctx, const double* const* V_dev, int m, const double* w_dev, int64_t n, int arith,
                   double* h_host);
/* EPSSetInitialSpace with one vector (normalised by the solver); on_device
 * selects whether v points to device or host memory.  NULL clears it. */
int ed_eps_set_initial_vector(ed_eps* e, const ed_cplx* v, int on_device);
/* Solver::solve: returns nconv. */
int ed_eps_solve(ed_eps* e, int* nconv);
/* Solver::solution(i): eigenvalue, relative error ||Hx - lx|| / |l|, and
 * (optionally) the eigenvector into a device or host buffer. */
int ed_eps_get_eigenpair(ed_eps* e, int i, double* eig, double* rel_err, ed_cplx* vec_dev);
int ed_eps_get_eigenvector_host(ed_eps* e, int i, ed_cplx* vec_host);
/* Iterations (restarts), H.v applications, eigenvalues reported, and
 * Gram-Schmidt update passes (one per step, two when refinement was needed). */
int ed_eps_get_stats(ed_eps* e, int* its, int64_t* n_hv, int* n_reported, int64_t* ortho_passes);
int ed_eps_destroy(ed_eps* e);  /* Solver::SolverClean */

/* ---- batched disorder sweep: replaces the one-realisation-at-a-time loop
 *      of examples/main_disorder.cpp:82-120 -------------------------------- */
typedef struct ed_batch ed_batch;
/* B realisations of h (uniform J1/J2, build_off_diag done) with fields
 * hi_host[b*N + i]; each realisation's diagonal is build_disorder's
 * (hamiltonian.tmpl_func.hpp:97-125), bit for bit.  Vectors of the batch are
 * [dim][B] complex128 (realisation index fastest). */
int ed_batch_create(ed_ham* h, int B, const double* hi_host, ed_batch** out);
int ed_batch_destroy(ed_batch* bt);
/* Y[:, b] = H_b X[:, b] for every realisation. */
int ed_batch_apply(ed_batch* bt, const ed_cplx* x_dev, ed_cplx* y_dev);
/* The [dim][B] diagonal (MatGetDiagonal per realisation). */
int ed_batch_diag_host(ed_batch* bt, double* out_host);
/* Lowest nev eigenpairs of every realisation by lockstep Krylov-Schur (same
 * method and start vector as ed_eps_solve); evals/errs [B][nev], nconv [B]. */
int ed_batch_solve(ed_batch* bt, int nev, int ncv, double tol, int max_it, uint64_t seed, double* evals_host,
                   double* errs_host, int* nconv_host);
/* Eigenvector i of realisation b into a contiguous device vector. */
int ed_batch_get_eigenvector(ed_batch* bt, int b, int i, ed_cplx* vec_dev);
int ed_batch_stats(ed_batch* bt, int* its, int64_t* n_hv);
/* Several batched sweeps at once (e.g. the Sz sectors of one disorder
 * sweep): bts[i] is solved as by ed_batch_solve into evals_host[i] /
 * errs_host[i] / nconv_host[i], each on its own host thread.  Every batch
 * must belong to a different environment (its own stream), so that the
 * device overlaps them.  Returns the first error, prefixed with the batch's
 * index.  No counterpart in the reference (its sectors run one after
 * another). */
int ed_batch_solve_many(ed_batch* const* bts, int count, int nev, int ncv, double tol, int max_it, uint64_t seed,
                        double* const* evals_host, double* const* errs_host, int* const* nconv_host);
/* CUDA graphs for the batched solve: with on != 0 (the default), every
 * expansion sweep after the first (which tunes the batched H.v and sizes the
 * buffers) is captured from the batch's stream into a CUDA graph and
 * launched from it.  The sweep has no host round trip, so the graph holds
 * all of its kernels; the results are those of direct launches bit for bit.
 * A sweep's columns change at every restart, so each graph is captured and
 * instantiated once.  on = 0 launches the kernels directly.
 * ed_batch_graph_sweeps reports how many sweeps of the last solve ran from
 * a graph.  No counterpart in the reference. */
int ed_batch_set_graphs(ed_batch* bt, int on);
int ed_batch_graph_sweeps(const ed_batch* bt, int64_t* n);
/* Tile of the batched H.v: rows of the basis per CTA tile (4, 8, 16, 32)
 * and threads per CTA (128, 256; the realisation columns are spread over
 * them).  (0, 0) re-enables the autotuner, which times every tile once at the
 * batch's first real-storage H.v and keeps the fastest.  All tiles give
 * bit-identical H.v results; the x^T y and ||y||^2 fused into the solve's
 * H.v are summed per tile, so a solve's last bits can depend on the tile.
 * No counterpart in the reference. */
int ed_batch_set_hv_tile(ed_batch* bt, int rows, int threads);
/* The tile in use ((0, 0) before the autotuner has run). */
int ed_batch_hv_tile(const ed_batch* bt, int* rows, int* threads);
/* Products of the restart combination, as ed_eps_set_restart_arithmetic. */
int ed_batch_set_restart_arithmetic(ed_batch* bt, int mode);

/* ---- measurements: replace SiSj/SzSz/SpSm/SmSp::ExpectVal
 *      (src/spinOperators/correlation.cpp:38-299) --------------------------- */
/* out[p] = ExpectVal(op, i_p, j_p, psi) for npairs pairs, 16 per pass over
 * the basis (PETSc VecDot convention: sum_s psi_s * conj((O psi)_s)).  For a
 * real psi (every imaginary part zero, as the solver's eigenvectors), the
 * S^z S^z part and the one-site sums are exact integer sums of the FP64
 * weights psi_s^2 rounded once, and the call holds a temporary copy of the
 * real parts (8 * dim bytes) on the device; without room for it, or for a
 * non-finite psi, the general FP64 kernel runs instead. */
int ed_expect_pairs(const ed_basis* b, int op, const ed_cplx* psi_dev, const int32_t* pairs_host,
                    int64_t npairs, ed_cplx* out_host);
/* All N*N <S_i.S_j> (op = ED_OP_SISJ) into out_host[i*N + j]. */
int ed_expect_all_pairs(const ed_basis* b, int op, const ed_cplx* psi_dev, ed_cplx* out_host);

/* ---- DSF: replaces Phys::DynStructFactor's coefficient loop
 *      (include/phys.tmpl_func.hpp:161-186) --------------------------------- */
/* c[i*nev + n] = VecDot(S_i |psi0>, v_n) = v_n^H S_i psi0, for all sites i
 * and nev target vectors v_n (device, column n at vecs_dev + n*dim1).
 * op 0 = Sqz (same sector, spinOPft.tmpl_func.hpp:28-60),
 * op 1 = Sqp (S+ into sector m+1, spinOPft.tmpl_func.hpp:77-143). */
int ed_dsf_coefficients(const ed_basis* b0, const ed_basis* b1, int op, const ed_cplx* psi0_dev,
                        const ed_cplx* vecs_dev, int nev, ed_cplx* c_host);
/* S(q, w) from DSF coefficients, replacing the post-processing notebook
 * (postprocessing/dynamicStep0_preprocess.ipynb cells 11-15):
 * S_dev[iq*nw + k] += sum_n F[iq][n] * (1/pi) eps^2 / (eps^2 + (w_k - dE[n])^2),
 * F[iq][n] = |sum_i exp(i q.r_i) c[i*nev + n]|^2 / nspins, w_k = w_min + k (w_max - w_min)/(nw - 1),
 * q_host[2*iq..] = (q_x, q_y), r_host[2*i..] = site position.  S_dev (device,
 * nq x nw doubles) accumulates, so disorder realisations sum in place; the
 * notebook's average is then 2 pi / rep times the sum (cell 17). */
int ed_dsf_spectrum(ed_ctx* ctx, int nspins, int nev, const ed_cplx* c_host, const double* dE_host, int nq,
                    const double* q_host, const double* r_host, int nw, double w_min, double w_max, double eps,
                    double* S_dev);

/* ---- disorder: replaces Tools::RandomDisorder
 *      (src/tools/random_disorder.cpp:33-59), host only --------------------- */
/* srand_seq_init: rep seeds ~ uniform_int(0, 1000) from mt19937_64(1) when
 * reprod != 0, else from std::random_device. */
int ed_random_seeds(int reprod, int64_t rep, int64_t* seeds_host);
/* hi_init: h_i ~ uniform_real(min, max) from mt19937_64(seed), i < nspins. */
int ed_random_fields(int64_t seed, int nspins, double min, double max, double* hi_host);
/* n draws of std::normal_distribution(0, 1) from mt19937_64(seed) (per-bond
 * coupling disorder; no counterpart in the reference). */
int ed_random_normal(int64_t seed, int64_t n, double* out_host);

/* ---- adjoint gradients: no counterpart in the reference (uniform couplings,
 *      no derivatives).  H = sum_b [J_b XY_b + D_b ZZ_b] + sum_i h_i Z_i with
 *      XY_b = (S+_i S-_j + S-_i S+_j)/2, ZZ_b = S^z_i S^z_j, Z_i = S^z_i. ---- */
enum { ED_TERM_XY = 0, ED_TERM_ZZ = 1, ED_TERM_Z = 2, ED_TERM_SISJ = 3 };
/* out[t] = <lam| O_t |psi> for terms (kind[t], ij[2t], ij[2t+1]); Z ignores j;
 * XY and SISJ with i == j give the identity/2 and S.S = 3/4 respectively. */
int ed_expect_mixed(const ed_basis* b, const int* kinds_host, const int32_t* ij_host, int64_t nterms,
                    const ed_cplx* lam_dev, const ed_cplx* psi_dev, ed_cplx* out_host);
/* out = O psi for one term (no aliasing). */
int ed_apply_term(const ed_basis* b, int kind, int i, int j, const ed_cplx* psi_dev, ed_cplx* out_dev);
/* Hellmann-Feynman gradient of E = <psi|H|psi>/<psi|psi> for an eigenvector
 * psi: dJ[q] = <XY_q>, dD[q] = <ZZ_q> for bond q = (pairs[2q], pairs[2q+1]),
 * dh[i] = <S^z_i>.  Any output may be NULL. */
int ed_grad_energy(const ed_basis* b, const int32_t* pairs_host, int64_t nbonds, const ed_cplx* psi_dev,
                   double* dJ_host, double* dD_host, double* dh_host);
/* MINRES for (H - shift) x = rhs, projected onto the complement of the unit
 * vector q_dev (NULL: no projection).  Stops at ||r|| <= tol ||rhs||. */
int ed_minres(ed_ham* h, double shift, const ed_cplx* rhs_dev, const ed_cplx* q_dev, double tol, int max_it,
              ed_cplx* x_dev, int* its_out, double* relres_out);

#ifdef __cplusplus
}
#endif
#endif /* ED_CAPI_H */
