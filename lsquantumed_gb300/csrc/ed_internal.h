// Internal declarations shared by the libedgb300 translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "../../include/ed_capi.h"

#define ED_MAX_BONDS 256
#define ED_MAX_TYPES 256
#define ED_MAX_SPINS 32
#define ED_RANK_MAX_CHUNKS 4

// ---------------------------------------------------------------------------
// Error state (thread local) and helpers.
// ---------------------------------------------------------------------------
void ed_set_error(const std::string& msg);
int ed_fail(int code, const std::string& msg);
int ed_cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define ED_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess) return ed_cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)
#define ED_CHECK_LAUNCH(ctx)                                                  \
  do {                                                                        \
    cudaError_t _e = cudaGetLastError();                                      \
    if (_e != cudaSuccess) return ed_cuda_fail(_e, "kernel launch", __FILE__, __LINE__); \
    (ctx)->kernels++;                                                         \
  } while (0)
#define ED_TRY(expr)            \
  do {                          \
    int _rc = (expr);           \
    if (_rc != ED_OK) return _rc; \
  } while (0)

// ---------------------------------------------------------------------------
// Combinadic rank tables.  The N-bit state is split into K chunks (bottom to
// top, widths w[k] at bit offsets off[k]).  rank(s) = sum_k T_k[c_k][chunk_k]
// where c_k = number of set bits below chunk k; T_0 is indexed by the chunk
// only (c = 0) and the top chunk's c is fixed by nup - popc(top chunk).  Each
// entry is sum over the chunk's set bits (t-th from the bottom) of
// C(off + q, c + t) — the combinadic sum of src/hamiltonian.cpp:9-27 split by
// chunks, exact in integers.
// ---------------------------------------------------------------------------
struct RankTables {
  int K;                          // number of chunks (1..4)
  int nup;
  int w[ED_RANK_MAX_CHUNKS];      // chunk widths
  int off[ED_RANK_MAX_CHUNKS];    // bit offset of each chunk
  int base[ED_RANK_MAX_CHUNKS];   // entry offset of each chunk's table
  int total;                      // total entries
  const uint32_t* tab;            // device pointer (total entries)
};

// Bonds in the order the reference visits them, with coupling types.
// mask = (1 << i) | (1 << j); type indexes the per-type coefficients.
// For the incremental rank: a bond (i, j), i < j, lies in chunks ci <= cj
// of the rank tables; flipping it changes only the table entries of chunks
// ci..cj (the chunk values of ci and cj, and the set-bit count below every
// chunk in (ci, cj]).  xm[b][k] is the bond's mask restricted to chunk k.
struct BondSet {
  int nb;
  int ntypes;
  int per_bond;                   // 1: one type per bond (J_b, D_b)
  uint32_t mask[ED_MAX_BONDS];
  uint8_t type[ED_MAX_BONDS];
  uint8_t ci[ED_MAX_BONDS], cj[ED_MAX_BONDS], lo[ED_MAX_BONDS];
  uint16_t xm[ED_MAX_BONDS][ED_RANK_MAX_CHUNKS];
  double chalf[ED_MAX_TYPES];     // J_t * 0.5 (off-diagonal element per bond)
};

// Bonds regrouped for the fixed-point H.v kernel: segments by (chunk class
// (ci, cj), coupling type); each bond packed as
// mask | xm[ci] << 32 | xm[cj] << 48.  Segment s = (class * 2 + type) spans
// word[seg[s] .. seg[s+1]).  Classes enumerate (ci, cj), ci <= cj, row-major.
#define ED_NCLASS 10
struct BondSegments {
  int seg[2 * ED_NCLASS + 1];
  unsigned long long word[ED_MAX_BONDS];
};

struct ed_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t kernels = 0;
  // reduction scratch (device) and pinned host mirror
  double* d_red = nullptr;
  size_t red_cap = 0;             // doubles
  double* h_red = nullptr;
  int reduce_blocks = 0;
  // H.v launch timing (events on the stream)
  bool profiling = false;
  std::vector<cudaEvent_t> prof_events;  // pairs (start, stop)
};

struct ed_basis {
  ed_ctx* ctx = nullptr;
  int nspins = 0, nup = 0, total_mag = 0;
  int64_t dim = 0;
  uint32_t* d_states = nullptr;
  RankTables rt{};
  uint32_t* d_tab = nullptr;
  std::vector<uint32_t> h_tab;    // host copy of the rank tables
  // two-table rank: rank(s) = lin_t0[s & (2^lin_w0 - 1)] + lin_t1[s >> lin_w0]
  int lin_w0 = 0;
  uint16_t* d_lin_t0 = nullptr;
  uint32_t* d_lin_t1 = nullptr;
};

struct ed_lin;  // two-table fixed-point H.v state (ed_hv_lin.cu)

struct ed_ham {
  ed_ctx* ctx = nullptr;
  const ed_basis* basis = nullptr;
  // batched H.v tile chosen by the autotuner, per batch width (ed_batch.cu)
  std::vector<std::pair<int, int>> batch_tile;
  // neighbour table of the run-time compiled H.v (ed_hv_jit.cu): t1[c1 ^ m1]
  // per high half c1 in the module's slot order; jit_t1n_key is the module
  void* jit_t1n = nullptr;
  const void* jit_t1n_key = nullptr;
  // reference parameters (uniform mode)
  bool per_bond = false;
  double J1 = 0, D1 = 0, J2 = 0, D2 = 0;
  std::vector<int32_t> bi, bj;    // ordered bonds (nn first, then nnn in uniform mode)
  std::vector<int> btype;         // 0 = nn, 1 = nnn (uniform) / bond index (per-bond)
  std::vector<double> bJ, bD;     // per-bond couplings (per-bond mode)
  int n_nn = 0;
  bool diag_built = false, offdiag_built = false, disorder = false;
  std::vector<double> hi;
  double* d_diag = nullptr;       // assembled diagonal
  BondSet bs{};                   // off-diagonal bond set (empty until build_off_diag)
  int mode = ED_HAM_MATRIX_FREE;
  // explicit CSR (real values; H is real symmetric)
  int64_t* d_rowptr = nullptr;
  uint32_t* d_cols = nullptr;
  double* d_vals = nullptr;
  int64_t nnz = 0;
  // scratch for the host-buffer apply
  double2* d_x = nullptr;
  double2* d_y = nullptr;
  // block floating point copy of the H.v input (integer accumulation path)
  longlong2* d_xq = nullptr;      // 62-bit mantissas, (re, im) per state
  uint16_t* d_xe = nullptr;       // biased exponent per 32-state block
  int* d_gmax = nullptr;          // largest block exponent
  // d_xq / d_gmax already hold the fixed-point copy of this real vector
  // (ed_scale_quantize_r); the next two-table H.v of it uses them once
  const void* xq_src = nullptr;
  int hv_kernel = 2;              // 0: FP64, 1: exact 128-bit, 2: 64-bit fixed point
  BondSegments segs{};
  ed_lin* lin = nullptr;          // tables and bond words of the two-table kernel
};

// ---------------------------------------------------------------------------
// Launchers implemented in the .cu files.
// ---------------------------------------------------------------------------
int ed_build_rank_tables(int nspins, int nup, RankTables& rt, std::vector<uint32_t>& tab);
// Two-table rank for b (ed_hv_lin.cu): fills b->lin_w0, d_lin_t0, d_lin_t1.
int ed_basis_lin_tables(ed_basis* b);
int ed_launch_basis_states(ed_ctx* ctx, int nspins, int nup, int64_t dim, uint32_t* states);
int ed_launch_rank(ed_ctx* ctx, const ed_basis* b, const uint32_t* states_dev, int64_t n, int64_t* ranks_dev);
int ed_launch_unrank(ed_ctx* ctx, const ed_basis* b, const int64_t* ranks_dev, int64_t n, uint32_t* states_dev);

int ed_launch_build_diag(ed_ham* h);
int ed_launch_hv(ed_ham* h, const double2* x, double2* y);
// y = H x and, in the same pass over the rows, dot = x^H y and *y2 = ||y||^2.
// Returns ED_ENOTSUP (nothing launched) where the operator has no fused form.
int ed_launch_hv_dot(ed_ham* h, const double2* x, double2* y, double2* dot, double* y2);
// Same for x, y complex (rio false) or real storage double[dim] (rio true).
int ed_launch_hv_dot_any(ed_ham* h, const void* x, void* y, bool rio, double2* dot, double* y2);
// y = H x with real storage (two-table kernel only).
int ed_launch_hv_r(ed_ham* h, const double* x, double* y);
// Fixed-point copy of x into h->d_xq: largest exponent, non-finite flag and
// imaginary-nonzero flag in h->d_gmax[0..2]; when every imaginary part is
// zero only the real parts are stored (int64[dim]).  *sbits = the scale.
int ed_fx64_quantize(ed_ham* h, const double2* x, int* sbits);
int ed_fx64_quantize_r(ed_ham* h, const double* x, int* sbits);
// Largest biased exponent among fl(v_r * s), given absmax_hi = max_r |v_r|
// with its low 32 bits cleared (the device tracks the high words only).  The
// true maximum lies between absmax_hi and absmax_hi with the low word all
// ones, and rounding is monotonic, so the exponent is known when both bounds
// give the same one; -1 otherwise (or when not finite, or s <= 0).
int ed_fx64_emax_scaled(double absmax_hi, double s);
// dst = src * s (real storage) and, in the same pass, dst's fixed-point copy
// for the next H.v of dst (h->xq_src = dst), bit-identical to what
// ed_fx64_quantize_r would make of dst.  src_absmax_hi as above.  Returns
// ED_ENOTSUP without launching anything when the exponent is not determined.
int ed_scale_quantize_r(ed_ham* h, const double* src, double* dst, double s, double src_absmax_hi);
// sbits of h's fixed-point H.v input (depends on the bond counts only).
int ed_fx64_sbits(const ed_ham* h);
bool ed_lin_supported(const ed_ham* h);
// rio: x and y are real storage (double[dim]) instead of complex128.
int ed_launch_hv_lin(ed_ham* h, const void* x, void* y, bool dot, int* nblk_out, bool rio);
// The two-table H.v compiled at run time for one operator's bond words
// (ed_hv_jit.cu); ED_ENOTSUP where no run-time compiler is available.
// budget 0, 1, 2: register budget for 2, 4 or 3 blocks of 256 per SM; 3, 4:
// one block of 768 or 1024 per SM.
// coef (nullable): per-bond coefficients of the words (the per-bond form),
// on the host (passed as a launch parameter) and in device memory (coef_dev,
// read by the checked path); the row sums are then scaled by 2^pbexp.
int ed_jit_launch(ed_ham* h, uint64_t signature, int budget, const void* x, void* y, bool dot, int sbits,
                  int* nblk_out, const unsigned long long* words, const int* seg, int w0, bool rio,
                  const long long* coef = nullptr, const long long* coef_dev = nullptr, int pbexp = 0);
// NVRTC and the driver entry points can be loaded (the run-time compiled
// kernels can exist at all).
bool ed_jit_available();
void ed_lin_invalidate(ed_lin* L);
const char* ed_lin_variant_name(const ed_ham* h, int dot);
int ed_lin_set_variant(ed_ham* h, const char* name);
void ed_lin_free(ed_lin* L);
int ed_launch_csr_build(ed_ham* h);
int ed_launch_csr_spmv(ed_ham* h, const double2* x, double2* y);
void ed_ham_make_bondset(ed_ham* h);
// Unique-mask coefficients for the assembled matrix (duplicates summed in
// the reference's ADD_VALUES order).
void ed_ham_unique_masks(const ed_ham* h, std::vector<uint32_t>& masks, std::vector<double>& vals);

// linear algebra on device vectors (complex128)
int ed_ensure_reduce(ed_ctx* ctx, size_t doubles);
// Sum `items` rows of nblk per-block partials in ctx->d_red (fixed order),
// copy to host_out and synchronise the stream.
// The last nmax items are maximised over the blocks instead of summed.
int ed_finish_reduce(ed_ctx* ctx, int items, int nblk, double* host_out, int nmax = 0);
int ed_start_vector(ed_ctx* ctx, uint64_t seed, int64_t n, double2* v, bool real_only = false);
// *real = every imaginary part of v is zero.
int ed_is_real(ed_ctx* ctx, const double2* v, int64_t n, bool* real);
// real = true: V and w are real (imaginary parts exactly zero); only the
// real parts are formed (imaginary parts of the results returned as 0).
int ed_multidot(ed_ctx* ctx, const double2* const* cols, int nv, const double2* w, int64_t n,
                double2* h_host, double* wnorm2_host, bool real = false);
// real = true: all vectors and coefficients are real (imaginary parts exactly
// zero: H real symmetric and a real start vector); only real parts are formed.
int ed_update(ed_ctx* ctx, const double2* const* cols, int nv, const double2* h_host, double2* w, int64_t n,
              double* wnorm2_host, bool real = false);
int ed_local_multidot(ed_ctx* ctx, const double2* const* cols, int nv, double2* w, int64_t n, const double2* vj,
                      double2 a, const double2* vjm1, double b, double2* h_host, double* wnorm2_host, bool real = false);
int ed_scale_copy(ed_ctx* ctx, const double2* src, double2* dst, double s, int64_t n);
int ed_restart_combine(ed_ctx* ctx, const double2* const* cols, int m, const double* Y, int ldY, int l,
                       double2* const* out, int64_t n, bool real = false);
int ed_residual_norm2(ed_ctx* ctx, const double2* hx, const double2* x, double theta, int64_t n, double* r2_host,
                      double* x2_host);
int ed_copy(ed_ctx* ctx, const double2* src, double2* dst, int64_t n);
// Real storage (real-mode solves keep only the real parts of the basis).
int ed_multidot_r(ed_ctx* ctx, const double* const* cols, int nv, double* w, int64_t n, const double* vj, double a,
                  const double* vjm1, double b, double* h_host, double* wnorm2_host);
// wmax_host (nullable): max_r |w_r| after the update with its low 32 bits
// cleared (see ed_fx64_emax_scaled).
// arith: ED_RESTART_FIXED forms sum_i V_i h_i on the integer units (exact
// products of 56-bit fixed-point inputs, one rounding per row), otherwise
// FP64 FMAs.
int ed_update_r(ed_ctx* ctx, const double* const* cols, int nv, const double* h_host, double* w, int64_t n,
                double* wnorm2_host, double* wmax_host = nullptr, int arith = ED_RESTART_FP64);
int ed_scale_copy_r(ed_ctx* ctx, const double* src, double* dst, double s, int64_t n);
// arith: ED_RESTART_FP64 (FP64 FMA beside exact integer products),
// ED_RESTART_PAIR (float-pair products on the FP32 units, ed_linalg.cu) or
// ED_RESTART_EXACT (exact slices on the tensor cores, ed_tc.cu; m <= 32).
int ed_restart_combine_r(ed_ctx* ctx, const double* const* cols, int m, const double* Y, int ldY, int l,
                         double* const* out, int64_t n, int arith = ED_RESTART_FP64);
// h_host[i] = V_i^T w (i < nv) on the tensor cores in exact slices
// (ed_tc.cu); with vj the local step w <- w - a vj - b vjm1 first (written
// back).  wbound: an upper bound on max |w| after the local step; ED_ENOTSUP
// when it did not hold (the local step is then done, the dots are not).
int ed_multidot_tc(ed_ctx* ctx, const double* const* cols, int nv, double* w, int64_t n, const double* vj, double a,
                   const double* vjm1, double b, double wbound, double* h_host);
// out_c = sum_i V_i Y[i][c], c < l, on the tensor cores in exact slices
// (ed_tc.cu).  ED_ENOTSUP (nothing launched) for m outside 1..32.
int ed_restart_combine_tc(ed_ctx* ctx, const double* const* cols, int m, const double* Y, int ldY, int l,
                          double* const* out, int64_t n);
int ed_residual_norm2_r(ed_ctx* ctx, const double* hx, const double* x, double theta, int64_t n, double* r2_host,
                        double* x2_host);
int ed_start_vector_r(ed_ctx* ctx, uint64_t seed, int64_t n, double* v);
int ed_real_to_complex(ed_ctx* ctx, const double* src, double2* dst, int64_t n);
int ed_complex_to_real(ed_ctx* ctx, const double2* src, double* dst, int64_t n);

// measurements
int ed_launch_expect_pairs(const ed_basis* b, int op, const double2* psi, const int32_t* pairs_host, int64_t np,
                           double2* out_host);
int ed_launch_dsf(const ed_basis* b0, const ed_basis* b1, int op, const double2* psi0, const double2* vecs, int nev,
                  double2* c_host);

// small dense symmetric eigensolver (host)
void ed_jacobi_eig(int m, std::vector<double>& A, std::vector<double>& theta, std::vector<double>& Y);

uint64_t ed_binom(int n, int k);
