// C ABI entry points: context, basis, lattice, Hamiltonian, measurements.
// The eigensolver entry points live in ed_eps.cu.
#include "ed_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>

static thread_local std::string g_err;

void ed_set_error(const std::string& msg) { g_err = msg; }
int ed_fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int ed_cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  const char* base = strrchr(file, '/');  // the source file's name, not the build machine's path
  base = base ? base + 1 : file;
  g_err = std::string("CUDA error: ") + cudaGetErrorString(e) + " in " + what + " (" + base + ":" + std::to_string(line) + ")";
  return e == cudaErrorMemoryAllocation ? ED_ENOMEM : ED_ECUDA;
}

extern "C" {

int ed_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return (int)g_err.size();
  size_t n = std::min(len - 1, g_err.size());
  memcpy(buf, g_err.data(), n);
  buf[n] = 0;
  return (int)g_err.size();
}

int ed_version(void) { return 1; }

// ---------------------------------------------------------------------------
// Context (Environment, src/environment.cpp:8-49, without MPI)
// ---------------------------------------------------------------------------
int ed_ctx_create(int device, void* stream, ed_ctx** out) {
  if (!out) return ed_fail(ED_EINVAL, "null output");
  int ndev = 0;
  ED_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0) ED_CUDA(cudaGetDevice(&device));
  if (device >= ndev) return ed_fail(ED_EINVAL, "device index out of range");
  ED_CUDA(cudaSetDevice(device));
  ed_ctx* c = new ed_ctx();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) { delete c; return ed_cuda_fail(e, "cudaDeviceGetAttribute", __FILE__, __LINE__); }
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return ed_cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__); }
    c->own_stream = true;
  }
  *out = c;
  return ED_OK;
}

static void clear_profile(ed_ctx* c) {
  for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
  c->prof_events.clear();
}

int ed_ctx_profile(ed_ctx* c, int enable) {
  if (!c) return ed_fail(ED_EINVAL, "null context");
  ED_CUDA(cudaStreamSynchronize(c->stream));
  clear_profile(c);
  c->profiling = enable != 0;
  return ED_OK;
}

int ed_ctx_profile_read(ed_ctx* c, int64_t* n_hv, double* ms_hv) {
  if (!c) return ed_fail(ED_EINVAL, "null context");
  ED_CUDA(cudaStreamSynchronize(c->stream));
  double tot = 0.0;
  for (size_t k = 0; k + 1 < c->prof_events.size(); k += 2) {
    float ms = 0.f;
    ED_CUDA(cudaEventElapsedTime(&ms, c->prof_events[k], c->prof_events[k + 1]));
    tot += ms;
  }
  if (n_hv) *n_hv = (int64_t)(c->prof_events.size() / 2);
  if (ms_hv) *ms_hv = tot;
  return ED_OK;
}

int ed_ctx_destroy(ed_ctx* c) {
  if (!c) return ED_OK;
  cudaStreamSynchronize(c->stream);
  clear_profile(c);
  if (c->d_red) cudaFree(c->d_red);
  if (c->h_red) cudaFreeHost(c->h_red);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  delete c;
  return ED_OK;
}

int ed_ctx_synchronize(ed_ctx* c) {
  if (!c) return ed_fail(ED_EINVAL, "null context");
  ED_CUDA(cudaStreamSynchronize(c->stream));
  return ED_OK;
}

int ed_ctx_kernel_count(const ed_ctx* c, int64_t* count) {
  if (!c || !count) return ed_fail(ED_EINVAL, "null argument");
  *count = c->kernels;
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Device vectors
// ---------------------------------------------------------------------------
int ed_vec_create(ed_ctx* ctx, int64_t n, ed_cplx** vec_dev) {
  if (!ctx || !vec_dev || n < 0) return ed_fail(ED_EINVAL, "bad argument");
  ED_CUDA(cudaSetDevice(ctx->device));
  void* p = nullptr;
  if (cudaMalloc(&p, sizeof(ed_cplx) * (size_t)std::max<int64_t>(n, 1)) != cudaSuccess) {
    cudaGetLastError();
    return ed_fail(ED_ENOMEM, "vector does not fit in device memory");
  }
  *vec_dev = (ed_cplx*)p;
  return ED_OK;
}

int ed_vec_destroy(ed_cplx* vec_dev) {
  if (vec_dev) cudaFree(vec_dev);
  return ED_OK;
}

int ed_vec_to_host(ed_ctx* ctx, const ed_cplx* vec_dev, ed_cplx* host, int64_t n) {
  if (!ctx || ((!vec_dev || !host) && n > 0) || n < 0) return ed_fail(ED_EINVAL, "bad argument");
  if (n == 0) return ED_OK;
  ED_CUDA(cudaMemcpyAsync(host, vec_dev, sizeof(ed_cplx) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  return ED_OK;
}

int ed_vec_from_host(ed_ctx* ctx, const ed_cplx* host, ed_cplx* vec_dev, int64_t n) {
  if (!ctx || ((!vec_dev || !host) && n > 0) || n < 0) return ed_fail(ED_EINVAL, "bad argument");
  if (n == 0) return ED_OK;
  ED_CUDA(cudaMemcpyAsync(vec_dev, host, sizeof(ed_cplx) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Basis (src/basis.cpp:56-94)
// ---------------------------------------------------------------------------
static int64_t compute_size(int nspins, int nup) {
  // basis.cpp:38-46
  double size = 1.0;
  for (int64_t i = 1; i <= (nspins - nup); ++i) size *= ((double)(i + nup) / (double)i);
  return (int64_t)std::floor(size + 0.5);
}

int ed_basis_create(ed_ctx* ctx, int nspins, int total_mag, ed_basis** out) {
  if (!ctx || !out) return ed_fail(ED_EINVAL, "null argument");
  if (nspins % 2 != 0) return ed_fail(ED_EINVAL, "The total number of spins has to be EVEN.");
  if (nspins <= 0) return ed_fail(ED_EINVAL, "The total number of spins has to be POSITIVE.");
  if (total_mag > nspins / 2 || total_mag < -nspins / 2)
    return ed_fail(ED_EINVAL, "The required constant magnetization has to be <= nspins/2.");
  if (nspins > ED_MAX_SPINS) return ed_fail(ED_ENOTSUP, "the device path supports nspins <= 32");
  ED_CUDA(cudaSetDevice(ctx->device));
  ed_basis* b = new ed_basis();
  b->ctx = ctx;
  b->nspins = nspins;
  b->total_mag = total_mag;
  b->nup = total_mag + nspins / 2;
  b->dim = compute_size(nspins, b->nup);
  int rc = ed_build_rank_tables(nspins, b->nup, b->rt, b->h_tab);
  if (rc != ED_OK) { delete b; return rc; }
  cudaError_t e1 = cudaMalloc(&b->d_states, sizeof(uint32_t) * (size_t)b->dim);
  cudaError_t e2 = cudaMalloc(&b->d_tab, sizeof(uint32_t) * (size_t)b->rt.total);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaGetLastError();
    if (b->d_states) cudaFree(b->d_states);
    if (b->d_tab) cudaFree(b->d_tab);
    delete b;
    return ed_fail(ED_ENOMEM, "basis does not fit in device memory");
  }
  b->rt.tab = b->d_tab;
  cudaError_t e3 = cudaMemcpyAsync(b->d_tab, b->h_tab.data(), sizeof(uint32_t) * b->h_tab.size(), cudaMemcpyHostToDevice,
                                   ctx->stream);
  if (e3 != cudaSuccess) { ed_basis_destroy(b); return ed_cuda_fail(e3, "upload rank tables", __FILE__, __LINE__); }
  rc = ed_launch_basis_states(ctx, nspins, b->nup, b->dim, b->d_states);
  if (rc != ED_OK) { ed_basis_destroy(b); return rc; }
  rc = ed_basis_lin_tables(b);
  if (rc != ED_OK) { ed_basis_destroy(b); return rc; }
  *out = b;
  return ED_OK;
}

// Destroy functions do not touch the context (it may already be gone when a
// garbage-collecting host language finalises objects out of order); cudaFree
// waits for outstanding work on the buffers.
int ed_basis_destroy(ed_basis* b) {
  if (!b) return ED_OK;
  if (b->d_states) cudaFree(b->d_states);
  if (b->d_tab) cudaFree(b->d_tab);
  if (b->d_lin_t0) cudaFree(b->d_lin_t0);
  if (b->d_lin_t1) cudaFree(b->d_lin_t1);
  delete b;
  return ED_OK;
}

int ed_basis_info(const ed_basis* b, int64_t* size, int* nspins, int* nspins_up, int* total_mag) {
  if (!b) return ed_fail(ED_EINVAL, "null basis");
  if (size) *size = b->dim;
  if (nspins) *nspins = b->nspins;
  if (nspins_up) *nspins_up = b->nup;
  if (total_mag) *total_mag = b->total_mag;
  return ED_OK;
}

int ed_basis_states_host(const ed_basis* b, int64_t start, int64_t count, uint64_t* out_host) {
  if (!b || (!out_host && count > 0)) return ed_fail(ED_EINVAL, "null argument");
  if (start < 0 || count < 0 || start + count > b->dim) return ed_fail(ED_EINVAL, "state range out of bounds");
  if (count == 0) return ED_OK;
  std::vector<uint32_t> tmp((size_t)count);
  ED_CUDA(cudaMemcpyAsync(tmp.data(), b->d_states + start, sizeof(uint32_t) * (size_t)count, cudaMemcpyDeviceToHost,
                          b->ctx->stream));
  ED_CUDA(cudaStreamSynchronize(b->ctx->stream));
  for (int64_t i = 0; i < count; ++i) out_host[i] = tmp[(size_t)i];
  return ED_OK;
}

int ed_basis_rank_host(const ed_basis* b, const uint64_t* states_host, int64_t* ranks_host, int64_t n) {
  if (!b || ((!states_host || !ranks_host) && n > 0)) return ed_fail(ED_EINVAL, "null argument");
  if (n <= 0) return ED_OK;
  std::vector<uint32_t> s((size_t)n);
  const uint64_t lim = b->nspins == 32 ? 0xFFFFFFFFull : ((1ull << b->nspins) - 1);
  for (int64_t i = 0; i < n; ++i) {
    uint64_t v = states_host[i];
    if (v > lim || __builtin_popcountll(v) != b->nup)
      return ed_fail(ED_EINVAL, "state " + std::to_string(v) + " is not in this fixed-Sz sector");
    s[(size_t)i] = (uint32_t)v;
  }
  ed_ctx* ctx = b->ctx;
  uint32_t* ds = nullptr;
  int64_t* dr = nullptr;
  ED_CUDA(cudaMalloc(&ds, sizeof(uint32_t) * (size_t)n));
  ED_CUDA(cudaMalloc(&dr, sizeof(int64_t) * (size_t)n));
  ED_CUDA(cudaMemcpyAsync(ds, s.data(), sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = ed_launch_rank(ctx, b, ds, n, dr);
  if (rc == ED_OK) {
    cudaMemcpyAsync(ranks_host, dr, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = ed_cuda_fail(e, "rank", __FILE__, __LINE__);
  }
  cudaFree(ds);
  cudaFree(dr);
  return rc;
}

int ed_basis_unrank_host(const ed_basis* b, const int64_t* ranks_host, uint64_t* states_host, int64_t n) {
  if (!b || ((!states_host || !ranks_host) && n > 0)) return ed_fail(ED_EINVAL, "null argument");
  if (n <= 0) return ED_OK;
  for (int64_t i = 0; i < n; ++i)
    if (ranks_host[i] < 0 || ranks_host[i] >= b->dim) return ed_fail(ED_EINVAL, "rank out of range");
  ed_ctx* ctx = b->ctx;
  uint32_t* ds = nullptr;
  int64_t* dr = nullptr;
  ED_CUDA(cudaMalloc(&ds, sizeof(uint32_t) * (size_t)n));
  ED_CUDA(cudaMalloc(&dr, sizeof(int64_t) * (size_t)n));
  ED_CUDA(cudaMemcpyAsync(dr, ranks_host, sizeof(int64_t) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = ed_launch_unrank(ctx, b, dr, n, ds);
  std::vector<uint32_t> s((size_t)n);
  if (rc == ED_OK) {
    cudaMemcpyAsync(s.data(), ds, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = ed_cuda_fail(e, "unrank", __FILE__, __LINE__);
    for (int64_t i = 0; i < n; ++i) states_host[i] = s[(size_t)i];
  }
  cudaFree(ds);
  cudaFree(dr);
  return rc;
}

int ed_basis_device_states(const ed_basis* b, const uint32_t** states_dev) {
  if (!b || !states_dev) return ed_fail(ED_EINVAL, "null argument");
  *states_dev = b->d_states;
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Lattice bonds (src/lattice.cpp:27-264), flattened in visiting order.
// ---------------------------------------------------------------------------
int ed_lattice_bonds(int ltype, int nspins, int lx, int ly, int32_t* nn_pairs, int64_t nn_cap, int64_t* n_nn,
                     int32_t* nnn_pairs, int64_t nnn_cap, int64_t* n_nnn) {
  if (nspins <= 0) return ed_fail(ED_EINVAL, "nspins must be positive");
  std::vector<int32_t> a, b;
  if (ltype == ED_CHAIN1D) {
    for (int i = 0; i < nspins; ++i) { a.push_back(i); a.push_back((i + 1) % nspins); }
    for (int i = 0; i < nspins; ++i) { b.push_back(i); b.push_back((i + 2) % nspins); }
  } else if (ltype == ED_SQUARE2D || ltype == ED_HONEYCOMB2D) {
    if ((int64_t)lx * ly != nspins || lx <= 0 || ly <= 0)
      return ed_fail(ED_EINVAL, "The product between the number of spins in x direction and the numer of spins in the y "
                                "direction has to be equal to the total number of spins.");
    if (ltype == ED_SQUARE2D) {
      for (int ix = 0; ix < lx; ++ix)
        for (int iy = 0; iy < ly; ++iy) {
          int c = ix * ly + iy;
          a.push_back(c); a.push_back(ix * ly + (iy + 1) % ly);
          a.push_back(c); a.push_back(((ix + 1) % lx) * ly + iy);
        }
      for (int ix = 0; ix < lx; ++ix)
        for (int iy = 0; iy < ly; ++iy) {
          int c = ix * ly + iy;
          b.push_back(c); b.push_back(((ix + 1) % lx) * ly + (iy + 1) % ly);
          b.push_back(c); b.push_back(((ix + 1) % lx) * ly + (iy - 1 + ly) % ly);
        }
    } else {
      if (lx % 2 != 0 || ly % 2 != 0) return ed_fail(ED_EINVAL, "The number of spins in each direction has to be even.");
      for (int ix = 0; ix < lx; ++ix)
        for (int iy = 0; iy < ly; ++iy) {
          int c = ix * ly + iy;
          bool two = (ix % 2 == 0) ? (c % 2 == 0) : (c % 2 != 0);
          a.push_back(c); a.push_back(ix * ly + (iy + 1) % ly);
          if (two) { a.push_back(c); a.push_back(((ix + 1) % lx) * ly + iy); }
        }
      for (int ix = 0; ix < lx; ++ix)
        for (int iy = 0; iy < ly; ++iy) {
          int c = ix * ly + iy;
          b.push_back(c); b.push_back(ix * ly + (iy + 2) % ly);
          b.push_back(c); b.push_back(((ix + 1) % lx) * ly + (iy + 1) % ly);
          b.push_back(c); b.push_back(((ix + 1) % lx) * ly + (iy - 1 + ly) % ly);
        }
    }
  } else {
    return ed_fail(ED_EINVAL, "unknown lattice type");
  }
  int64_t na = (int64_t)a.size() / 2, nb = (int64_t)b.size() / 2;
  if (n_nn) *n_nn = na;
  if (n_nnn) *n_nnn = nb;
  if (nn_pairs) {
    if (nn_cap < na) return ed_fail(ED_EINVAL, "nn capacity too small");
    std::copy(a.begin(), a.end(), nn_pairs);
  }
  if (nnn_pairs) {
    if (nnn_cap < nb) return ed_fail(ED_EINVAL, "nnn capacity too small");
    std::copy(b.begin(), b.end(), nnn_pairs);
  }
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Hamiltonian (include/hamiltonian.hpp:187-249)
// ---------------------------------------------------------------------------
static int ham_alloc(ed_ctx* ctx, const ed_basis* b, ed_ham* h) {
  h->ctx = ctx;
  h->basis = b;
  if (cudaMalloc(&h->d_diag, sizeof(double) * (size_t)b->dim) != cudaSuccess) {
    cudaGetLastError();
    return ed_fail(ED_ENOMEM, "diagonal does not fit in device memory");
  }
  ED_CUDA(cudaMemsetAsync(h->d_diag, 0, sizeof(double) * (size_t)b->dim, ctx->stream));
  return ED_OK;
}

static int check_pairs(const ed_basis* b, const int32_t* p, int64_t n) {
  if (n > 0 && !p) return ed_fail(ED_EINVAL, "null bond list");
  for (int64_t k = 0; k < 2 * n; ++k)
    if (p[k] < 0 || p[k] >= b->nspins) return ed_fail(ED_EINVAL, "bond site index out of range");
  return ED_OK;
}

int ed_ham_create(ed_ctx* ctx, const ed_basis* b, const int32_t* nn_pairs, int64_t n_nn, const int32_t* nnn_pairs,
                  int64_t n_nnn, double J1, double D1, double J2, double D2, ed_ham** out) {
  if (!ctx || !b || !out) return ed_fail(ED_EINVAL, "null argument");
  if (n_nn < 0 || n_nnn < 0 || n_nn + n_nnn > ED_MAX_BONDS) return ed_fail(ED_ENOTSUP, "at most 256 bonds");
  ED_TRY(check_pairs(b, nn_pairs, n_nn));
  ED_TRY(check_pairs(b, nnn_pairs, n_nnn));
  ed_ham* h = new ed_ham();
  h->J1 = J1; h->D1 = D1; h->J2 = J2; h->D2 = D2;
  for (int64_t k = 0; k < n_nn; ++k) { h->bi.push_back(nn_pairs[2 * k]); h->bj.push_back(nn_pairs[2 * k + 1]); h->btype.push_back(0); }
  for (int64_t k = 0; k < n_nnn; ++k) { h->bi.push_back(nnn_pairs[2 * k]); h->bj.push_back(nnn_pairs[2 * k + 1]); h->btype.push_back(1); }
  h->n_nn = (int)n_nn;
  int rc = ham_alloc(ctx, b, h);
  if (rc != ED_OK) { delete h; return rc; }
  *out = h;
  return ED_OK;
}

int ed_ham_create_bonds(ed_ctx* ctx, const ed_basis* b, const int32_t* pairs, int64_t nbonds, const double* J_host,
                        const double* D_host, ed_ham** out) {
  if (!ctx || !b || !out || (nbonds > 0 && (!J_host || !D_host))) return ed_fail(ED_EINVAL, "null argument");
  if (nbonds < 0 || nbonds > ED_MAX_BONDS) return ed_fail(ED_ENOTSUP, "at most 256 bonds");
  ED_TRY(check_pairs(b, pairs, nbonds));
  ed_ham* h = new ed_ham();
  h->per_bond = true;
  for (int64_t k = 0; k < nbonds; ++k) {
    h->bi.push_back(pairs[2 * k]); h->bj.push_back(pairs[2 * k + 1]); h->btype.push_back((int)k);
    h->bJ.push_back(J_host[k]); h->bD.push_back(D_host[k]);
  }
  int rc = ham_alloc(ctx, b, h);
  if (rc != ED_OK) { delete h; return rc; }
  *out = h;
  return ED_OK;
}

static void ham_free_csr(ed_ham* h) {
  if (h->d_rowptr) cudaFree(h->d_rowptr);
  if (h->d_cols) cudaFree(h->d_cols);
  if (h->d_vals) cudaFree(h->d_vals);
  h->d_rowptr = nullptr; h->d_cols = nullptr; h->d_vals = nullptr; h->nnz = 0;
}

int ed_ham_destroy(ed_ham* h) {
  if (!h) return ED_OK;
  if (h->d_diag) cudaFree(h->d_diag);
  if (h->d_x) cudaFree(h->d_x);
  if (h->d_y) cudaFree(h->d_y);
  if (h->d_xq) cudaFree(h->d_xq);
  if (h->jit_t1n) cudaFree(h->jit_t1n);
  if (h->d_xe) cudaFree(h->d_xe);
  if (h->d_gmax) cudaFree(h->d_gmax);
  ed_lin_free(h->lin);
  ham_free_csr(h);
  delete h;
  return ED_OK;
}

int ed_ham_build_diag(ed_ham* h) {
  if (!h) return ed_fail(ED_EINVAL, "null Hamiltonian");
  h->diag_built = true;
  if (h->d_rowptr) ham_free_csr(h);
  return ed_launch_build_diag(h);
}

int ed_ham_build_off_diag(ed_ham* h) {
  if (!h) return ed_fail(ED_EINVAL, "null Hamiltonian");
  h->offdiag_built = true;
  if (h->d_rowptr) ham_free_csr(h);
  ed_ham_make_bondset(h);
  return ED_OK;
}

int ed_ham_build_disorder(ed_ham* h, const double* hi_host) {
  if (!h || !hi_host) return ed_fail(ED_EINVAL, "null argument");
  h->disorder = true;
  h->hi.assign(hi_host, hi_host + h->basis->nspins);
  if (h->d_rowptr) ham_free_csr(h);
  return ed_launch_build_diag(h);
}

int ed_ham_apply(ed_ham* h, const ed_cplx* x_dev, ed_cplx* y_dev) {
  if (!h || !x_dev || !y_dev) return ed_fail(ED_EINVAL, "null argument");
  if (x_dev == y_dev) return ed_fail(ED_EINVAL, "x and y must not alias");
  return ed_launch_hv(h, (const double2*)x_dev, (double2*)y_dev);
}

int ed_ham_apply_real(ed_ham* h, const double* x_dev, double* y_dev) {
  if (!h || !x_dev || !y_dev) return ed_fail(ED_EINVAL, "null argument");
  if (x_dev == y_dev) return ed_fail(ED_EINVAL, "x and y must not alias");
  return ed_launch_hv_r(h, x_dev, y_dev);
}

int ed_bv_mult_real(ed_ctx* ctx, const double* const* V_dev, int m, const double* Y_host, int ldY, int l,
                    double* const* out_dev, int64_t n, int arith) {
  if (!ctx || !V_dev || !Y_host || !out_dev) return ed_fail(ED_EINVAL, "null argument");
  if (m < 1 || l < 1 || n < 1 || ldY < l) return ed_fail(ED_EINVAL, "bad dimensions");
  if (m > 127 || l > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  for (int i = 0; i < m; ++i)
    for (int c = 0; c < l; ++c)
      if (V_dev[i] == out_dev[c]) return ed_fail(ED_EINVAL, "out must not alias V");
  if (arith == ED_RESTART_AUTO) arith = ED_RESTART_FP64;
  if (arith != ED_RESTART_FP64 && arith != ED_RESTART_PAIR && arith != ED_RESTART_EXACT &&
      arith != ED_RESTART_FIXED)
    return ed_fail(ED_EINVAL, "unknown restart arithmetic");
  if (arith == ED_RESTART_EXACT && m > 32) return ed_fail(ED_ENOTSUP, "the exact restart takes at most 32 vectors");
  ED_CUDA(cudaSetDevice(ctx->device));
  return ed_restart_combine_r(ctx, V_dev, m, Y_host, ldY, l, out_dev, n, arith);
}

int ed_bv_dot_real(ed_ctx* ctx, const double* const* V_dev, int m, const double* w_dev, int64_t n, int arith,
                   double* h_host) {
  if (!ctx || !V_dev || !w_dev || !h_host) return ed_fail(ED_EINVAL, "null argument");
  if (m < 1 || n < 1) return ed_fail(ED_EINVAL, "bad dimensions");
  if (m > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  if (arith == ED_RESTART_AUTO) arith = ED_RESTART_FP64;
  if (arith != ED_RESTART_FP64 && arith != ED_RESTART_EXACT) return ed_fail(ED_EINVAL, "unknown dot arithmetic");
  ED_CUDA(cudaSetDevice(ctx->device));
  double* w = const_cast<double*>(w_dev);  // read only: no local step
  if (arith == ED_RESTART_EXACT) {
    double w2 = 0.0;
    ED_TRY(ed_multidot_r(ctx, nullptr, 0, w, n, nullptr, 0.0, nullptr, 0.0, nullptr, &w2));
    const double bound = std::sqrt(w2) * (1.0 + 0x1p-40);
    if (bound > 0.0) {
      const int rc = ed_multidot_tc(ctx, V_dev, m, w, n, nullptr, 0.0, nullptr, 0.0, bound, h_host);
      if (rc != ED_ENOTSUP) return rc;
    }
  }
  return ed_multidot_r(ctx, V_dev, m, w, n, nullptr, 0.0, nullptr, 0.0, h_host, nullptr);
}

int ed_ham_apply_real_dot(ed_ham* h, const double* x_dev, double* y_dev, double* xy_host, double* yy_host) {
  if (!h || !x_dev || !y_dev) return ed_fail(ED_EINVAL, "null argument");
  if (x_dev == y_dev) return ed_fail(ED_EINVAL, "x and y must not alias");
  if (!ed_lin_supported(h)) return ed_fail(ED_ENOTSUP, "real-storage H.v needs the two-table fixed-point kernel");
  double2 dot;
  double y2 = 0.0;
  ED_TRY(ed_launch_hv_dot_any(h, x_dev, y_dev, true, &dot, &y2));
  if (xy_host) *xy_host = dot.x;
  if (yy_host) *yy_host = y2;
  return ED_OK;
}

int ed_ham_apply_host(ed_ham* h, const ed_cplx* x_host, ed_cplx* y_host) {
  if (!h || !x_host || !y_host) return ed_fail(ED_EINVAL, "null argument");
  ed_ctx* ctx = h->ctx;
  const size_t bytes = sizeof(double2) * (size_t)h->basis->dim;
  if (!h->d_x) ED_CUDA(cudaMalloc(&h->d_x, bytes));
  if (!h->d_y) ED_CUDA(cudaMalloc(&h->d_y, bytes));
  ED_CUDA(cudaMemcpyAsync(h->d_x, x_host, bytes, cudaMemcpyHostToDevice, ctx->stream));
  ED_TRY(ed_launch_hv(h, h->d_x, h->d_y));
  ED_CUDA(cudaMemcpyAsync(y_host, h->d_y, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  return ED_OK;
}

int ed_ham_build_csr(ed_ham* h, int64_t* nnz) {
  if (!h) return ed_fail(ED_EINVAL, "null Hamiltonian");
  ED_TRY(ed_launch_csr_build(h));
  if (nnz) *nnz = h->nnz;
  return ED_OK;
}

int ed_ham_set_mode(ed_ham* h, int mode) {
  if (!h) return ed_fail(ED_EINVAL, "null Hamiltonian");
  if (mode != ED_HAM_MATRIX_FREE && mode != ED_HAM_CSR) return ed_fail(ED_EINVAL, "unknown mode");
  if (mode == ED_HAM_CSR && !h->d_rowptr) ED_TRY(ed_launch_csr_build(h));
  h->mode = mode;
  return ED_OK;
}

int ed_ham_export_csr_host(ed_ham* h, int64_t* rowptr_host, int64_t* cols_host, double* vals_host, int64_t cap) {
  if (!h || !rowptr_host) return ed_fail(ED_EINVAL, "null argument");
  if (!h->d_rowptr) ED_TRY(ed_launch_csr_build(h));
  if (cap < h->nnz || ((!cols_host || !vals_host) && h->nnz > 0))
    return ed_fail(ED_EINVAL, "export capacity " + std::to_string(cap) + " < nnz " + std::to_string(h->nnz));
  ed_ctx* ctx = h->ctx;
  const int64_t dim = h->basis->dim;
  std::vector<uint32_t> c((size_t)h->nnz);
  ED_CUDA(cudaMemcpyAsync(rowptr_host, h->d_rowptr, sizeof(int64_t) * (size_t)(dim + 1), cudaMemcpyDeviceToHost, ctx->stream));
  if (h->nnz > 0) {
    ED_CUDA(cudaMemcpyAsync(c.data(), h->d_cols, sizeof(uint32_t) * (size_t)h->nnz, cudaMemcpyDeviceToHost, ctx->stream));
    ED_CUDA(cudaMemcpyAsync(vals_host, h->d_vals, sizeof(double) * (size_t)h->nnz, cudaMemcpyDeviceToHost, ctx->stream));
  }
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int64_t k = 0; k < h->nnz; ++k) cols_host[k] = c[(size_t)k];
  return ED_OK;
}

int ed_ham_diag_host(ed_ham* h, double* out_host) {
  if (!h || !out_host) return ed_fail(ED_EINVAL, "null argument");
  ED_CUDA(cudaMemcpyAsync(out_host, h->d_diag, sizeof(double) * (size_t)h->basis->dim, cudaMemcpyDeviceToHost,
                          h->ctx->stream));
  ED_CUDA(cudaStreamSynchronize(h->ctx->stream));
  return ED_OK;
}

int ed_ham_set_accumulation(ed_ham* h, int kind) {
  if (!h) return ed_fail(ED_EINVAL, "null Hamiltonian");
  if (kind != ED_ACC_FP64 && kind != ED_ACC_EXACT && kind != ED_ACC_FIXED64)
    return ed_fail(ED_EINVAL, "unknown accumulation kind");
  h->hv_kernel = kind;
  return ED_OK;
}

int ed_ham_size(const ed_ham* h, int64_t* size) {
  if (!h || !size) return ed_fail(ED_EINVAL, "null argument");
  *size = h->basis->dim;
  return ED_OK;
}

int ed_ham_set_hv_variant(ed_ham* h, const char* name) {
  if (!h || !name) return ed_fail(ED_EINVAL, "null argument");
  if (!ed_lin_supported(h)) return ed_fail(ED_ENOTSUP, "this operator does not use the two-table H.v");
  return ed_lin_set_variant(h, name);
}

int ed_ham_hv_variant(const ed_ham* h, int dot, char* buf, size_t len) {
  if (!h || !buf || len == 0) return ed_fail(ED_EINVAL, "null argument");
  const char* name = ed_lin_variant_name(h, dot);
  size_t n = strlen(name);
  if (n >= len) n = len - 1;
  memcpy(buf, name, n);
  buf[n] = 0;
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Measurements
// ---------------------------------------------------------------------------
int ed_expect_pairs(const ed_basis* b, int op, const ed_cplx* psi_dev, const int32_t* pairs_host, int64_t npairs,
                    ed_cplx* out_host) {
  if (!b || !psi_dev || (npairs > 0 && (!pairs_host || !out_host))) return ed_fail(ED_EINVAL, "null argument");
  if (op < ED_OP_SZSZ || op > ED_OP_SISJ) return ed_fail(ED_EINVAL, "unknown operator");
  for (int64_t k = 0; k < 2 * npairs; ++k)
    if (pairs_host[k] < 0 || pairs_host[k] >= b->nspins) return ed_fail(ED_EINVAL, "site index out of range");
  if (npairs == 0) return ED_OK;
  return ed_launch_expect_pairs(b, op, (const double2*)psi_dev, pairs_host, npairs, (double2*)out_host);
}

int ed_expect_all_pairs(const ed_basis* b, int op, const ed_cplx* psi_dev, ed_cplx* out_host) {
  if (!b || !psi_dev || !out_host) return ed_fail(ED_EINVAL, "null argument");
  const int N = b->nspins;
  // <O_ji> = conj(<O_ij>) for all four operators (S^z_i S^z_j and S_i.S_j are
  // Hermitian and symmetric in i, j; S+_j S-_i = (S+_i S-_j)^dagger, likewise
  // S-S+): evaluate i <= j and mirror.
  std::vector<int32_t> pairs;
  for (int i = 0; i < N; ++i)
    for (int j = i; j < N; ++j) { pairs.push_back(i); pairs.push_back(j); }
  const int64_t np = (int64_t)pairs.size() / 2;
  std::vector<ed_cplx> half(np);
  ED_TRY(ed_expect_pairs(b, op, psi_dev, pairs.data(), np, half.data()));
  for (int64_t k = 0; k < np; ++k) {
    const int i = pairs[2 * k], j = pairs[2 * k + 1];
    out_host[(size_t)i * N + j] = half[k];
    out_host[(size_t)j * N + i] = ed_cplx{half[k].re, -half[k].im};
  }
  return ED_OK;
}

int ed_dsf_coefficients(const ed_basis* b0, const ed_basis* b1, int op, const ed_cplx* psi0_dev, const ed_cplx* vecs_dev,
                        int nev, ed_cplx* c_host) {
  if (!b0 || !b1 || !psi0_dev || !vecs_dev || !c_host) return ed_fail(ED_EINVAL, "null argument");
  if (nev < 1) return ed_fail(ED_EINVAL, "nev must be >= 1");
  if (b0->nspins != b1->nspins) return ed_fail(ED_EINVAL, "bases must have the same number of spins");
  if (op == 0 && b1->nup != b0->nup) return ed_fail(ED_EINVAL, "Sqz maps a sector onto itself");
  if (op == 1 && b1->nup != b0->nup + 1) return ed_fail(ED_EINVAL, "Sqp maps sector m onto m+1");
  if (op != 0 && op != 1) return ed_fail(ED_EINVAL, "unknown DSF operator");
  return ed_launch_dsf(b0, b1, op, (const double2*)psi0_dev, (const double2*)vecs_dev, nev, (double2*)c_host);
}

// ---------------------------------------------------------------------------
// Disorder generators (src/tools/random_disorder.cpp:33-59); PetscInt is
// 64-bit in the reference build.
// ---------------------------------------------------------------------------
int ed_random_seeds(int reprod, int64_t rep, int64_t* seeds_host) {
  if (rep < 0 || (rep > 0 && !seeds_host)) return ed_fail(ED_EINVAL, "bad argument");
  std::uniform_int_distribution<int64_t> dist(0, 1000);
  if (!reprod) {
    std::random_device rd;
    std::mt19937_64 g(rd());
    for (int64_t i = 0; i < rep; ++i) seeds_host[i] = dist(g);
  } else {
    std::mt19937_64 g(1);
    for (int64_t i = 0; i < rep; ++i) seeds_host[i] = dist(g);
  }
  return ED_OK;
}

int ed_random_fields(int64_t seed, int nspins, double mn, double mx, double* hi_host) {
  if (nspins < 0 || (nspins > 0 && !hi_host)) return ed_fail(ED_EINVAL, "bad argument");
  std::mt19937_64 g((uint64_t)seed);
  std::uniform_real_distribution<double> dist(mn, mx);
  for (int i = 0; i < nspins; ++i) hi_host[i] = dist(g);
  return ED_OK;
}

int ed_random_normal(int64_t seed, int64_t n, double* out_host) {
  if (n < 0 || (n > 0 && !out_host)) return ed_fail(ED_EINVAL, "bad argument");
  std::mt19937_64 g((uint64_t)seed);
  std::normal_distribution<double> dist(0.0, 1.0);
  for (int64_t i = 0; i < n; ++i) out_host[i] = dist(g);
  return ED_OK;
}

}  // extern "C"
