// Adjoint gradients (no counterpart in the reference, which has uniform
// couplings only and no derivatives).
//
// With H = sum_b [J_b XY_b + D_b ZZ_b] + sum_i h_i Z_i, where
//   XY_b = (S+_i S-_j + S-_i S+_j)/2,  ZZ_b = S^z_i S^z_j,  Z_i = S^z_i,
// (the reference's J/2 off-diagonal, D*0.25*(+-1) diagonal and 0.5*(+-h_i)
// field terms), Hellmann-Feynman gives dE_n/dJ_b = <n|XY_b|n>,
// dE_n/dD_b = <n|ZZ_b|n>, dE_n/dh_i = <n|Z_i|n> for a non-degenerate level.
// For a ground-state expectation <O>, with (H - E0) lambda = P (O - <O>) psi0
// (P projects out psi0) solved by MINRES, d<O>/dtheta = -2 Re <lambda|dH/dtheta|psi0>.
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#define TERM_G 8

// term kinds
enum { T_XY = 0, T_ZZ = 1, T_Z = 2, T_SISJ = 3 };

struct TermGroup {
  int n;
  int kind[TERM_G];
  int32_t i[TERM_G], j[TERM_G];
};

// (O psi)_s for one term, at state s of rank r (psi gathered through ranks).
template <int K>
__device__ __forceinline__ double2 op_apply(int kind, int i, int j, uint32_t s, const double2* __restrict__ psi,
                                            const double2 ps, const uint32_t* stab, const RankTables& rt) {
  const uint32_t a = (s >> i) & 1u, b = (s >> j) & 1u;
  double2 out = make_double2(0.0, 0.0);
  if (kind == T_Z) {
    const double f = a ? 0.5 : -0.5;
    return make_double2(f * ps.x, f * ps.y);
  }
  if (kind == T_ZZ || kind == T_SISJ) {
    const double f = (a ^ b) ? -0.25 : 0.25;
    out.x = f * ps.x;
    out.y = f * ps.y;
  }
  if ((kind == T_XY || kind == T_SISJ) && i != j && a != b) {
    const uint32_t c = ed_rank<K>(s ^ ((1u << i) | (1u << j)), stab, rt);
    const double2 q = __ldg(&psi[c]);
    out.x = fma(0.5, q.x, out.x);
    out.y = fma(0.5, q.y, out.y);
  }
  if ((kind == T_XY || kind == T_SISJ) && i == j) {
    // (S+S- + S-S+)/2 on one site = 1/2
    out.x = fma(0.5, ps.x, out.x);
    out.y = fma(0.5, ps.y, out.y);
  }
  return out;
}

// partial[(2*g+c)*nblk + blk] = sum_s conj(lam_s) (O_g psi)_s
template <int K>
__global__ void __launch_bounds__(256) k_expect_mixed(const uint32_t* __restrict__ states, const double2* __restrict__ lam,
                                                      const double2* __restrict__ psi, int64_t dim, const RankTables rt,
                                                      const TermGroup tg, double* __restrict__ partial, int nblk) {
  extern __shared__ uint32_t stab[];
  ed_load_tables(stab, rt);
  double acc[2 * TERM_G];
#pragma unroll
  for (int k = 0; k < 2 * TERM_G; ++k) acc[k] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const uint32_t s = states[r];
    const double2 l = lam[r];
    const double2 p = psi[r];
#pragma unroll
    for (int g = 0; g < TERM_G; ++g) {
      if (g >= tg.n) break;
      const double2 o = op_apply<K>(tg.kind[g], tg.i[g], tg.j[g], s, psi, p, stab, rt);
      // conj(l) * o
      acc[2 * g] += fma(l.x, o.x, l.y * o.y);
      acc[2 * g + 1] += fma(l.x, o.y, -l.y * o.x);
    }
  }
  __shared__ double sh[2 * TERM_G * 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < 2 * TERM_G; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k * 32 + wid] = v;
  }
  __syncthreads();
  if (wid == 0) {
    for (int k = 0; k < 2 * TERM_G; ++k) {
      double v = lane < nw ? sh[k * 32 + lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) partial[(size_t)k * nblk + blockIdx.x] = v;
    }
  }
}

__global__ void k_sum_items(const double* __restrict__ partial, int nblk, double* __restrict__ out) {
  __shared__ double sh[256];
  double a = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) a += partial[(size_t)blockIdx.x * nblk + b];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

template <int K>
__global__ void __launch_bounds__(256) k_apply_op(const uint32_t* __restrict__ states, const double2* __restrict__ psi,
                                                  int64_t dim, const RankTables rt, int kind, int i, int j,
                                                  double2* __restrict__ out) {
  extern __shared__ uint32_t stab[];
  ed_load_tables(stab, rt);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride)
    out[r] = op_apply<K>(kind, i, j, states[r], psi, psi[r], stab, rt);
}

// out = sum_t c_t v_t (up to 4 terms, complex coefficients)
// out may alias any input (element r is read before it is written).
__global__ void k_lincomb(int nt, const double2* v0, const double2* v1, const double2* v2, const double2* v3,
                          double2 c0, double2 c1, double2 c2, double2 c3, double2* out, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double2 a = make_double2(0.0, 0.0);
    const double2* vs[4] = {v0, v1, v2, v3};
    const double2 cs[4] = {c0, c1, c2, c3};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      if (t < nt) {
        const double2 x = vs[t][r];
        a.x = fma(cs[t].x, x.x, fma(-cs[t].y, x.y, a.x));
        a.y = fma(cs[t].x, x.y, fma(cs[t].y, x.x, a.y));
      }
    }
    out[r] = a;
  }
}

static int lincomb(ed_ctx* ctx, int64_t n, double2* out, std::initializer_list<std::pair<double2, const double2*>> terms) {
  const double2* v[4] = {nullptr, nullptr, nullptr, nullptr};
  double2 c[4] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  int nt = 0;
  for (auto& t : terms) { c[nt] = t.first; v[nt] = t.second; ++nt; }
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_lincomb<<<g, 256, 0, ctx->stream>>>(nt, v[0], v[1], v[2], v[3], c[0], c[1], c[2], c[3], out, n);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

static inline double2 cr(double x) { return make_double2(x, 0.0); }

template <int K>
static int mixed_k(const ed_basis* b, const double2* lam, const double2* psi, const int* kinds, const int32_t* ij,
                   int64_t nt, double2* out) {
  ed_ctx* ctx = b->ctx;
  const int64_t dim = b->dim;
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((dim + 255) / 256, (int64_t)ctx->num_sms * 2));
  ED_TRY(ed_ensure_reduce(ctx, (size_t)2 * TERM_G * nblk + 2 * TERM_G + 8));
  size_t smem = (size_t)b->rt.total * sizeof(uint32_t);
  ED_CUDA(cudaFuncSetAttribute(k_expect_mixed<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(56 * 1024)));
  double* res = ctx->d_red + (size_t)2 * TERM_G * nblk;
  for (int64_t t0 = 0; t0 < nt; t0 += TERM_G) {
    TermGroup tg;
    memset(&tg, 0, sizeof(tg));
    tg.n = (int)std::min<int64_t>(TERM_G, nt - t0);
    for (int g = 0; g < tg.n; ++g) {
      tg.kind[g] = kinds[t0 + g];
      tg.i[g] = ij[2 * (t0 + g)];
      tg.j[g] = ij[2 * (t0 + g) + 1];
    }
    k_expect_mixed<K><<<nblk, 256, smem, ctx->stream>>>(b->d_states, lam, psi, dim, b->rt, tg, ctx->d_red, nblk);
    ED_CHECK_LAUNCH(ctx);
    k_sum_items<<<2 * TERM_G, 256, 0, ctx->stream>>>(ctx->d_red, nblk, res);
    ED_CHECK_LAUNCH(ctx);
    ED_CUDA(cudaMemcpyAsync(ctx->h_red, res, sizeof(double) * 2 * TERM_G, cudaMemcpyDeviceToHost, ctx->stream));
    ED_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int g = 0; g < tg.n; ++g) out[t0 + g] = make_double2(ctx->h_red[2 * g], ctx->h_red[2 * g + 1]);
  }
  return ED_OK;
}

static int mixed(const ed_basis* b, const double2* lam, const double2* psi, const int* kinds, const int32_t* ij,
                 int64_t nt, double2* out) {
  switch (b->rt.K) {
    case 1: return mixed_k<1>(b, lam, psi, kinds, ij, nt, out);
    case 2: return mixed_k<2>(b, lam, psi, kinds, ij, nt, out);
    case 3: return mixed_k<3>(b, lam, psi, kinds, ij, nt, out);
    default: return mixed_k<4>(b, lam, psi, kinds, ij, nt, out);
  }
}

template <int K>
static int apply_op_k(const ed_basis* b, int kind, int i, int j, const double2* psi, double2* out) {
  ed_ctx* ctx = b->ctx;
  size_t smem = (size_t)b->rt.total * sizeof(uint32_t);
  ED_CUDA(cudaFuncSetAttribute(k_apply_op<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(56 * 1024)));
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((b->dim + 255) / 256, (int64_t)ctx->num_sms * 4));
  k_apply_op<K><<<g, 256, smem, ctx->stream>>>(b->d_states, psi, b->dim, b->rt, kind, i, j, out);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

extern "C" {

int ed_expect_mixed(const ed_basis* b, const int* kinds_host, const int32_t* ij_host, int64_t nterms,
                    const ed_cplx* lam_dev, const ed_cplx* psi_dev, ed_cplx* out_host) {
  if (!b || !lam_dev || !psi_dev || (nterms > 0 && (!kinds_host || !ij_host || !out_host)))
    return ed_fail(ED_EINVAL, "null argument");
  for (int64_t t = 0; t < nterms; ++t) {
    if (kinds_host[t] < ED_TERM_XY || kinds_host[t] > ED_TERM_SISJ) return ed_fail(ED_EINVAL, "unknown term kind");
    if (ij_host[2 * t] < 0 || ij_host[2 * t] >= b->nspins || ij_host[2 * t + 1] < 0 || ij_host[2 * t + 1] >= b->nspins)
      return ed_fail(ED_EINVAL, "site index out of range");
  }
  if (nterms == 0) return ED_OK;
  return mixed(b, (const double2*)lam_dev, (const double2*)psi_dev, kinds_host, ij_host, nterms, (double2*)out_host);
}

int ed_apply_term(const ed_basis* b, int kind, int i, int j, const ed_cplx* psi_dev, ed_cplx* out_dev) {
  if (!b || !psi_dev || !out_dev) return ed_fail(ED_EINVAL, "null argument");
  if ((const void*)psi_dev == (const void*)out_dev) return ed_fail(ED_EINVAL, "input and output must not alias");
  if (kind < ED_TERM_XY || kind > ED_TERM_SISJ) return ed_fail(ED_EINVAL, "unknown term kind");
  if (i < 0 || i >= b->nspins || j < 0 || j >= b->nspins) return ed_fail(ED_EINVAL, "site index out of range");
  switch (b->rt.K) {
    case 1: return apply_op_k<1>(b, kind, i, j, (const double2*)psi_dev, (double2*)out_dev);
    case 2: return apply_op_k<2>(b, kind, i, j, (const double2*)psi_dev, (double2*)out_dev);
    case 3: return apply_op_k<3>(b, kind, i, j, (const double2*)psi_dev, (double2*)out_dev);
    default: return apply_op_k<4>(b, kind, i, j, (const double2*)psi_dev, (double2*)out_dev);
  }
}

int ed_grad_energy(const ed_basis* b, const int32_t* pairs_host, int64_t nbonds, const ed_cplx* psi_dev, double* dJ_host,
                   double* dD_host, double* dh_host) {
  if (!b || !psi_dev || (nbonds > 0 && !pairs_host)) return ed_fail(ED_EINVAL, "null argument");
  const int N = b->nspins;
  std::vector<int> kinds;
  std::vector<int32_t> ij;
  for (int64_t q = 0; q < nbonds; ++q) {
    kinds.push_back(ED_TERM_XY); ij.push_back(pairs_host[2 * q]); ij.push_back(pairs_host[2 * q + 1]);
    kinds.push_back(ED_TERM_ZZ); ij.push_back(pairs_host[2 * q]); ij.push_back(pairs_host[2 * q + 1]);
  }
  for (int i = 0; i < N; ++i) { kinds.push_back(ED_TERM_Z); ij.push_back(i); ij.push_back(i); }
  std::vector<ed_cplx> out(kinds.size());
  ED_TRY(ed_expect_mixed(b, kinds.data(), ij.data(), (int64_t)kinds.size(), psi_dev, psi_dev, out.data()));
  // <psi|psi> normalisation
  double2 nrm;
  double n2 = 0.0;
  ED_TRY(ed_multidot(b->ctx, nullptr, 0, (const double2*)psi_dev, b->dim, &nrm, &n2));
  const double inv = 1.0 / n2;
  for (int64_t q = 0; q < nbonds; ++q) {
    if (dJ_host) dJ_host[q] = out[2 * q].re * inv;
    if (dD_host) dD_host[q] = out[2 * q + 1].re * inv;
  }
  for (int i = 0; i < N; ++i)
    if (dh_host) dh_host[i] = out[2 * nbonds + i].re * inv;
  return ED_OK;
}

#define MR_CUDA(call)                                          \
  do {                                                         \
    cudaError_t _e = (call);                                   \
    if (_e != cudaSuccess) {                                   \
      rc = ed_cuda_fail(_e, #call, __FILE__, __LINE__);        \
      goto done;                                               \
    }                                                          \
  } while (0)

// MINRES (Paige & Saunders 1975, in the form of the Stanford SOL code) for
// (H - shift) x = rhs on the complement of a given unit vector q (psi0):
// every operator application is followed by the projection P = I - q q^H,
// so the singular direction of H - E0 never enters.  rhs must be orthogonal
// to q (it is projected once more here).
int ed_minres(ed_ham* h, double shift, const ed_cplx* rhs_dev, const ed_cplx* q_dev, double tol, int max_it,
              ed_cplx* x_dev, int* its_out, double* relres_out) {
  if (!h || !rhs_dev || !x_dev) return ed_fail(ED_EINVAL, "null argument");
  ed_ctx* ctx = h->ctx;
  const int64_t n = h->basis->dim;
  if (tol <= 0) tol = 1e-12;
  if (max_it <= 0) max_it = (int)std::min<int64_t>(10 * n, 100000);
  double2* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double2) * (size_t)n * 7) != cudaSuccess) {
    cudaGetLastError();
    return ed_fail(ED_ENOMEM, "MINRES workspace does not fit in device memory");
  }
  double2 *r1 = buf, *r2 = buf + n, *y = buf + 2 * n, *v = buf + 3 * n, *w = buf + 4 * n, *w1 = buf + 5 * n,
          *w2 = buf + 6 * n;
  double2* x = (double2*)x_dev;
  const double2* q = (const double2*)q_dev;
  int rc = ED_OK;
  auto project = [&](double2* z) -> int {
    if (!q) return ED_OK;
    double2 c;
    const double2* qq[1] = {q};
    ED_TRY(ed_multidot(ctx, qq, 1, z, n, &c, nullptr));
    return lincomb(ctx, n, z, {{cr(1.0), z}, {make_double2(-c.x, -c.y), q}});
  };
  auto nrm = [&](const double2* z, double* out) -> int {
    double2 d;
    return ed_multidot(ctx, nullptr, 0, z, n, &d, out);
  };
  double beta1 = 0.0, t = 0.0;
  int itn = 0;
  double oldb = 0.0, beta, dbar = 0.0, epsln = 0.0, phibar, cs = -1.0, sn = 0.0, rnorm = 0.0;
  MR_CUDA(cudaMemcpyAsync(r1, rhs_dev, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
  if ((rc = project(r1)) != ED_OK) goto done;
  if ((rc = nrm(r1, &t)) != ED_OK) goto done;
  beta1 = std::sqrt(t);
  MR_CUDA(cudaMemsetAsync(x, 0, sizeof(double2) * (size_t)n, ctx->stream));
  MR_CUDA(cudaMemsetAsync(w, 0, sizeof(double2) * (size_t)n, ctx->stream));
  MR_CUDA(cudaMemsetAsync(w2, 0, sizeof(double2) * (size_t)n, ctx->stream));
  MR_CUDA(cudaMemcpyAsync(r2, r1, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
  beta = beta1;
  phibar = beta1;
  rnorm = beta1;
  if (beta1 == 0.0) goto done;
  for (itn = 1; itn <= max_it; ++itn) {
    const double s = 1.0 / beta;
    if ((rc = lincomb(ctx, n, v, {{cr(s), r2}})) != ED_OK) goto done;
    if ((rc = ed_launch_hv(h, v, y)) != ED_OK) goto done;
    // y = (H - shift) v, projected; minus the previous Lanczos term
    if (itn >= 2) {
      if ((rc = lincomb(ctx, n, y, {{cr(1.0), y}, {cr(-shift), v}, {cr(-beta / oldb), r1}})) != ED_OK) goto done;
    } else {
      if ((rc = lincomb(ctx, n, y, {{cr(1.0), y}, {cr(-shift), v}})) != ED_OK) goto done;
    }
    if ((rc = project(y)) != ED_OK) goto done;
    double2 alfa;
    {
      const double2* vv[1] = {v};
      if ((rc = ed_multidot(ctx, vv, 1, y, n, &alfa, nullptr)) != ED_OK) goto done;
    }
    if ((rc = lincomb(ctx, n, y, {{cr(1.0), y}, {cr(-alfa.x / beta), r2}})) != ED_OK) goto done;
    {  // r1 <- r2, r2 <- y; the old r1 buffer becomes the next y
      double2* tmp = r1;
      r1 = r2;
      r2 = y;
      y = tmp;
    }
    oldb = beta;
    if ((rc = nrm(r2, &t)) != ED_OK) goto done;
    beta = std::sqrt(t);
    const double oldeps = epsln;
    const double delta = cs * dbar + sn * alfa.x;
    const double gbar = sn * dbar - cs * alfa.x;
    epsln = sn * beta;
    dbar = -cs * beta;
    double gamma = std::sqrt(gbar * gbar + beta * beta);
    gamma = std::max(gamma, 1e-300);
    cs = gbar / gamma;
    sn = beta / gamma;
    const double phi = cs * phibar;
    phibar = sn * phibar;
    // w1 <- w2, w2 <- w, w <- (v - oldeps w1 - delta w2) / gamma
    std::swap(w1, w2);  // w1 now holds the old w2
    std::swap(w2, w);   // w2 now holds the old w
    if ((rc = lincomb(ctx, n, w, {{cr(1.0 / gamma), v}, {cr(-oldeps / gamma), w1}, {cr(-delta / gamma), w2}})) != ED_OK)
      goto done;
    if ((rc = lincomb(ctx, n, x, {{cr(1.0), x}, {cr(phi), w}})) != ED_OK) goto done;
    rnorm = phibar;
    if (rnorm <= tol * beta1) break;
    if (beta == 0.0) break;
  }
  // rounding leaves components along q in x: remove them once at the end
  if (rc == ED_OK) rc = project(x);
done:
  if (its_out) *its_out = itn;
  if (relres_out) *relres_out = beta1 > 0 ? rnorm / beta1 : 0.0;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(buf);
  return rc;
}

}  // extern "C"
