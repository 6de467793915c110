// Vector kernels of the Krylov-Schur solver (complex128, device-resident).
// Reductions are two-stage with a fixed block count and a fixed tree order,
// so every result is bit-reproducible run to run.
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>

#define ED_RED_THREADS 256
#define ED_GROUP 8

struct ColPtrs {
  const double2* p[128];
};

static int red_blocks(ed_ctx* ctx, int64_t n) {
  int64_t b = (n + ED_RED_THREADS - 1) / ED_RED_THREADS;
  int64_t cap = (int64_t)ctx->num_sms * 4;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

int ed_ensure_reduce(ed_ctx* ctx, size_t doubles) {
  if (doubles <= ctx->red_cap) return ED_OK;
  if (ctx->d_red) cudaFree(ctx->d_red);
  if (ctx->h_red) cudaFreeHost(ctx->h_red);
  ctx->d_red = nullptr;
  ctx->h_red = nullptr;
  size_t cap = std::max<size_t>(doubles, 1 << 16);
  ED_CUDA(cudaMalloc(&ctx->d_red, cap * sizeof(double)));
  ED_CUDA(cudaMallocHost(&ctx->h_red, cap * sizeof(double)));
  ctx->red_cap = cap;
  return ED_OK;
}

// partial[item * nblk + blk]
template <int G, bool REAL>
__global__ void __launch_bounds__(ED_RED_THREADS) k_multidot(const ColPtrs cp, int v0, int ng, const double2* __restrict__ w,
                                                             int64_t n, int with_norm, double* __restrict__ partial,
                                                             int nblk) {
  double acc[2 * G + 1];
#pragma unroll
  for (int k = 0; k < 2 * G + 1; ++k) acc[k] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const double2 wv = w[r];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g < ng) {
        const double2 v = cp.p[v0 + g][r];
        if (REAL) {
          acc[2 * g] = fma(v.x, wv.x, acc[2 * g]);
        } else {
          acc[2 * g] = fma(v.x, wv.x, fma(v.y, wv.y, acc[2 * g]));
          acc[2 * g + 1] = fma(v.x, wv.y, fma(-v.y, wv.x, acc[2 * g + 1]));
        }
      }
    }
    if (with_norm) acc[2 * G] = REAL ? fma(wv.x, wv.x, acc[2 * G]) : fma(wv.x, wv.x, fma(wv.y, wv.y, acc[2 * G]));
  }
  __shared__ double sh[(2 * G + 1) * 32];
  ed_block_reduce<2 * G + 1>(acc, sh);
  if (threadIdx.x == 0) {
    // compile-time indices only: a runtime-indexed acc[] would live in local memory
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g < ng) {
        partial[(size_t)(2 * (v0 + g)) * nblk + blockIdx.x] = acc[2 * g];
        partial[(size_t)(2 * (v0 + g) + 1) * nblk + blockIdx.x] = REAL ? 0.0 : acc[2 * g + 1];
      }
    }
    if (with_norm) partial[(size_t)(2 * (v0 + ng)) * nblk + blockIdx.x] = acc[2 * G];
  }
}

// Second stage: out[item] = sum_b partial[item*nblk + b] (fixed order).
// Items below nsum are summed over the blocks, the others maximised.
__global__ void k_reduce_items(const double* __restrict__ partial, int nblk, double* __restrict__ out, int nsum) {
  __shared__ double sh[256];
  const int item = blockIdx.x;
  const bool mx = item >= nsum;
  double a = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    const double v = partial[(size_t)item * nblk + b];
    a = mx ? fmax(a, v) : a + v;
  }
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = mx ? fmax(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[item] = sh[0];
}

int ed_finish_reduce(ed_ctx* ctx, int items, int nblk, double* host_out, int nmax) {
  double* out_dev = ctx->d_red + (size_t)items * nblk;
  k_reduce_items<<<items, 256, 0, ctx->stream>>>(ctx->d_red, nblk, out_dev, items - nmax);
  ED_CHECK_LAUNCH(ctx);
  ED_CUDA(cudaMemcpyAsync(ctx->h_red, out_dev, sizeof(double) * items, cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < items; ++i) host_out[i] = ctx->h_red[i];
  return ED_OK;
}

static ColPtrs make_cols(const double2* const* cols, int nv) {
  ColPtrs c;
  for (int i = 0; i < 128; ++i) c.p[i] = nullptr;
  for (int i = 0; i < nv && i < 128; ++i) c.p[i] = cols[i];
  return c;
}

int ed_multidot(ed_ctx* ctx, const double2* const* cols, int nv, const double2* w, int64_t n, double2* h_host,
                double* wnorm2_host, bool real) {
  if (nv > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  const int nblk = red_blocks(ctx, n);
  const int items = 2 * nv + 1;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)items * nblk + items));
  ColPtrs cp = make_cols(cols, nv);
  int with_norm_done = 0;
  for (int v0 = 0; v0 < nv || !with_norm_done; v0 += ED_GROUP) {
    int ng = std::max(0, std::min(ED_GROUP, nv - v0));
    int last = (v0 + ED_GROUP >= nv);
    if (real)
      k_multidot<ED_GROUP, true><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, last, ctx->d_red, nblk);
    else
      k_multidot<ED_GROUP, false><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, last, ctx->d_red, nblk);
    ED_CHECK_LAUNCH(ctx);
    if (last) with_norm_done = 1;
  }
  std::vector<double> out(items);
  ED_TRY(ed_finish_reduce(ctx, items, nblk, out.data()));
  for (int i = 0; i < nv; ++i) { h_host[i].x = out[2 * i]; h_host[i].y = out[2 * i + 1]; }
  if (wnorm2_host) *wnorm2_host = out[2 * nv];
  return ED_OK;
}

// Local Lanczos projection fused with the first group of the full CGS dot
// products: w <- w - a v_j - b v_{j-1} (written back when `local` is set),
// then partial[i] = V_{v0+i}^H w and ||w||^2.
template <int G, bool REAL>
__global__ void __launch_bounds__(ED_RED_THREADS) k_local_multidot(const ColPtrs cp, int v0, int ng,
                                                                   double2* __restrict__ w, int64_t n, int local,
                                                                   const double2* __restrict__ vj, double2 a,
                                                                   const double2* __restrict__ vjm1, double b,
                                                                   int with_norm, double* __restrict__ partial, int nblk) {
  double acc[2 * G + 1];
#pragma unroll
  for (int k = 0; k < 2 * G + 1; ++k) acc[k] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double2 wv = w[r];
    if (local) {
      const double2 p = vj[r];
      if (REAL) {
        wv.x = fma(-a.x, p.x, wv.x);
      } else {
        wv.x = fma(-a.x, p.x, fma(a.y, p.y, wv.x));
        wv.y = fma(-a.x, p.y, fma(-a.y, p.x, wv.y));
      }
      if (vjm1) {
        const double2 q = vjm1[r];
        wv.x = fma(-b, q.x, wv.x);
        if (!REAL) wv.y = fma(-b, q.y, wv.y);
      }
      w[r] = wv;
    }
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g < ng) {
        const double2 v = cp.p[v0 + g][r];
        if (REAL) {
          acc[2 * g] = fma(v.x, wv.x, acc[2 * g]);
        } else {
          acc[2 * g] = fma(v.x, wv.x, fma(v.y, wv.y, acc[2 * g]));
          acc[2 * g + 1] = fma(v.x, wv.y, fma(-v.y, wv.x, acc[2 * g + 1]));
        }
      }
    }
    if (with_norm) acc[2 * G] = REAL ? fma(wv.x, wv.x, acc[2 * G]) : fma(wv.x, wv.x, fma(wv.y, wv.y, acc[2 * G]));
  }
  __shared__ double sh[(2 * G + 1) * 32];
  ed_block_reduce<2 * G + 1>(acc, sh);
  if (threadIdx.x == 0) {
    // compile-time indices only: a runtime-indexed acc[] would live in local memory
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g < ng) {
        partial[(size_t)(2 * (v0 + g)) * nblk + blockIdx.x] = acc[2 * g];
        partial[(size_t)(2 * (v0 + g) + 1) * nblk + blockIdx.x] = REAL ? 0.0 : acc[2 * g + 1];
      }
    }
    if (with_norm) partial[(size_t)(2 * (v0 + ng)) * nblk + blockIdx.x] = acc[2 * G];
  }
}

int ed_local_multidot(ed_ctx* ctx, const double2* const* cols, int nv, double2* w, int64_t n, const double2* vj,
                      double2 a, const double2* vjm1, double b, double2* h_host, double* wnorm2_host, bool real) {
  if (nv > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  const int nblk = red_blocks(ctx, n);
  const int items = 2 * nv + 1;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)items * nblk + items));
  ColPtrs cp = make_cols(cols, nv);
  // the norm item must be computed after the local update: it is produced by
  // the last group, which runs after the first (local) one on the stream
  const int ngroups = (nv + ED_GROUP - 1) / ED_GROUP;
  for (int gidx = 0; gidx < ngroups; ++gidx) {
    const int v0 = gidx * ED_GROUP;
    const int ng = std::min(ED_GROUP, nv - v0);
    const int last = gidx == ngroups - 1;
    if (real)
      k_local_multidot<ED_GROUP, true><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, gidx == 0, vj, a,
                                                                               vjm1, b, last, ctx->d_red, nblk);
    else
      k_local_multidot<ED_GROUP, false><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, gidx == 0, vj, a,
                                                                                vjm1, b, last, ctx->d_red, nblk);
    ED_CHECK_LAUNCH(ctx);
  }
  std::vector<double> out(items);
  ED_TRY(ed_finish_reduce(ctx, items, nblk, out.data()));
  for (int i = 0; i < nv; ++i) { h_host[i].x = out[2 * i]; h_host[i].y = out[2 * i + 1]; }
  if (wnorm2_host) *wnorm2_host = out[2 * nv];
  return ED_OK;
}

// w <- w - sum_i V_i h_i ; partial ||w||^2.  REAL: the vectors and the
// coefficients are real (all imaginary parts exactly zero), so only the
// real parts are formed: one FMA per element per vector, same values.
template <bool REAL>
__global__ void __launch_bounds__(ED_RED_THREADS) k_update(const ColPtrs cp, int nv, const double2* __restrict__ h,
                                                           double2* __restrict__ w, int64_t n, double* __restrict__ partial,
                                                           int nblk) {
  __shared__ double2 sh_h[128];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) sh_h[i] = h[i];
  __syncthreads();
  double acc[1] = {0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // two rows per thread and iteration: twice the loads in flight
  for (int64_t r0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r0 < n; r0 += 2 * stride) {
    const int64_t r1 = r0 + stride;
    const bool has1 = r1 < n;
    double2 w0 = w[r0];
    double2 w1 = has1 ? w[r1] : make_double2(0.0, 0.0);
#pragma unroll 4
    for (int i = 0; i < nv; ++i) {
      const double2* col = cp.p[i];
      const double2 v0 = col[r0];
      const double2 v1 = has1 ? col[r1] : make_double2(0.0, 0.0);
      const double2 c = sh_h[i];
      if (REAL) {
        w0.x = fma(-v0.x, c.x, w0.x);
        w1.x = fma(-v1.x, c.x, w1.x);
      } else {
        w0.x = fma(-v0.x, c.x, fma(v0.y, c.y, w0.x));
        w0.y = fma(-v0.x, c.y, fma(-v0.y, c.x, w0.y));
        w1.x = fma(-v1.x, c.x, fma(v1.y, c.y, w1.x));
        w1.y = fma(-v1.x, c.y, fma(-v1.y, c.x, w1.y));
      }
    }
    w[r0] = w0;
    acc[0] = REAL ? fma(w0.x, w0.x, acc[0]) : fma(w0.x, w0.x, fma(w0.y, w0.y, acc[0]));
    if (has1) {
      w[r1] = w1;
      acc[0] = REAL ? fma(w1.x, w1.x, acc[0]) : fma(w1.x, w1.x, fma(w1.y, w1.y, acc[0]));
    }
  }
  __shared__ double sh[32];
  ed_block_reduce<1>(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
}

int ed_update(ed_ctx* ctx, const double2* const* cols, int nv, const double2* h_host, double2* w, int64_t n,
              double* wnorm2_host, bool real) {
  if (nv > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  const int nblk = red_blocks(ctx, n);
  ED_TRY(ed_ensure_reduce(ctx, (size_t)nblk + 4 + 2 * 128));
  // h goes after the partials and the result slot, on a 16-byte boundary
  double2* h_dev = (double2*)(ctx->d_red + ((nblk + 2 + 1) & ~1));
  ED_CUDA(cudaMemcpyAsync(h_dev, h_host, sizeof(double2) * nv, cudaMemcpyHostToDevice, ctx->stream));
  ColPtrs cp = make_cols(cols, nv);
  if (real) k_update<true><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, nv, h_dev, w, n, ctx->d_red, nblk);
  else k_update<false><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, nv, h_dev, w, n, ctx->d_red, nblk);
  ED_CHECK_LAUNCH(ctx);
  double out = 0.0;
  ED_TRY(ed_finish_reduce(ctx, 1, nblk, &out));
  if (wnorm2_host) *wnorm2_host = out;
  return ED_OK;
}

__global__ void k_scale_copy(const double2* __restrict__ src, double2* __restrict__ dst, double s, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double2 v = src[r];
    dst[r] = make_double2(v.x * s, v.y * s);
  }
}

int ed_scale_copy(ed_ctx* ctx, const double2* src, double2* dst, double s, int64_t n) {
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_scale_copy<<<g, 256, 0, ctx->stream>>>(src, dst, s, n);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

int ed_copy(ed_ctx* ctx, const double2* src, double2* dst, int64_t n) {
  ED_CUDA(cudaMemcpyAsync(dst, src, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
  return ED_OK;
}

// out_c = sum_i V_i * Y[i*ldY + c], c in [c0, c0+nc), nc <= 8; Y real.
// REAL: the columns are real (imaginary parts exactly zero): real parts only.
template <bool REAL>
__global__ void __launch_bounds__(256) k_restart(const ColPtrs cp, int m, const double* __restrict__ Y, int ldY, int c0,
                                                 int nc, const ColPtrs outp, int64_t n) {
  extern __shared__ double shY[];  // m x 8
  for (int k = threadIdx.x; k < m * 8; k += blockDim.x) {
    int i = k / 8, c = k % 8;
    shY[k] = (c < nc) ? Y[(size_t)i * ldY + c0 + c] : 0.0;
  }
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double ar[8], ai[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) { ar[c] = 0.0; ai[c] = 0.0; }
    for (int i = 0; i < m; ++i) {
      const double2 v = cp.p[i][r];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const double y = shY[i * 8 + c];
        ar[c] = fma(v.x, y, ar[c]);
        if (!REAL) ai[c] = fma(v.y, y, ai[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (c < nc) ((double2*)outp.p[c0 + c])[r] = make_double2(ar[c], ai[c]);
  }
}

int ed_restart_combine(ed_ctx* ctx, const double2* const* cols, int m, const double* Y, int ldY, int l,
                       double2* const* out, int64_t n, bool real) {
  if (m > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  ColPtrs cp = make_cols(cols, m);
  ColPtrs op = make_cols((const double2* const*)out, l);
  double* dY = nullptr;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)m * ldY + 16));
  dY = ctx->d_red;
  ED_CUDA(cudaMemcpyAsync(dY, Y, sizeof(double) * (size_t)m * ldY, cudaMemcpyHostToDevice, ctx->stream));
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 4));
  size_t smem = sizeof(double) * (size_t)m * 8;
  for (int c0 = 0; c0 < l; c0 += 8) {
    int nc = std::min(8, l - c0);
    if (real) k_restart<true><<<g, 256, smem, ctx->stream>>>(cp, m, dY, ldY, c0, nc, op, n);
    else k_restart<false><<<g, 256, smem, ctx->stream>>>(cp, m, dY, ldY, c0, nc, op, n);
    ED_CHECK_LAUNCH(ctx);
  }
  return ED_OK;
}

// ||hx - theta x||^2 and ||x||^2
__global__ void __launch_bounds__(ED_RED_THREADS) k_residual(const double2* __restrict__ hx, const double2* __restrict__ x,
                                                             double theta, int64_t n, double* __restrict__ partial,
                                                             int nblk) {
  double acc[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const double2 a = hx[r], b = x[r];
    const double dr = fma(-theta, b.x, a.x), di = fma(-theta, b.y, a.y);
    acc[0] = fma(dr, dr, fma(di, di, acc[0]));
    acc[1] = fma(b.x, b.x, fma(b.y, b.y, acc[1]));
  }
  __shared__ double sh[64];
  ed_block_reduce<2>(acc, sh);
  if (threadIdx.x == 0) { partial[blockIdx.x] = acc[0]; partial[nblk + blockIdx.x] = acc[1]; }
}

int ed_residual_norm2(ed_ctx* ctx, const double2* hx, const double2* x, double theta, int64_t n, double* r2_host,
                      double* x2_host) {
  const int nblk = red_blocks(ctx, n);
  ED_TRY(ed_ensure_reduce(ctx, (size_t)2 * nblk + 2));
  k_residual<<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(hx, x, theta, n, ctx->d_red, nblk);
  ED_CHECK_LAUNCH(ctx);
  double out[2] = {0.0, 0.0};
  ED_TRY(ed_finish_reduce(ctx, 2, nblk, out));
  *r2_host = out[0];
  *x2_host = out[1];
  return ED_OK;
}

// Deterministic start vector: re, im ~ U[-1, 1) from a counter hash (same
// bits as the CPU oracle's start vector); real_only zeroes the imaginary parts.
__global__ void k_start_vector(uint64_t seed, int64_t n, int real_only, double2* __restrict__ v) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const uint64_t base = seed * 0xD1B54A32D192ED03ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t h1 = ed_splitmix64(base + 2 * (uint64_t)i);
    const uint64_t h2 = ed_splitmix64(base + 2 * (uint64_t)i + 1);
    const double u1 = (double)(h1 >> 11) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);
    v[i] = make_double2(2.0 * u1 - 1.0, real_only ? 0.0 : 2.0 * u2 - 1.0);
  }
}

int ed_start_vector(ed_ctx* ctx, uint64_t seed, int64_t n, double2* v, bool real_only) {
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_start_vector<<<g, 256, 0, ctx->stream>>>(seed, n, real_only ? 1 : 0, v);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

// *any = 1 if some entry of v has a nonzero imaginary part.
__global__ void k_imag_any(const double2* __restrict__ v, int64_t n, int* __restrict__ any) {
  int a = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) a |= v[i].y != 0.0;
  a = (int)__reduce_or_sync(0xffffffffu, (unsigned)a);
  if ((threadIdx.x & 31) == 0 && a) atomicOr(any, 1);
}

int ed_is_real(ed_ctx* ctx, const double2* v, int64_t n, bool* real) {
  int* d_any = nullptr;
  ED_CUDA(cudaMalloc(&d_any, sizeof(int)));
  int h_any = 0;
  cudaError_t e = cudaMemsetAsync(d_any, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess) {
    int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
    k_imag_any<<<g, 256, 0, ctx->stream>>>(v, n, d_any);
    e = cudaGetLastError();
    if (e == cudaSuccess) ctx->kernels++;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_any, d_any, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_any);
  if (e != cudaSuccess) return ed_cuda_fail(e, "imaginary-part test", __FILE__, __LINE__);
  *real = h_any == 0;
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Real storage.  A Krylov basis grown by a real symmetric H from a real start
// vector has exactly zero imaginary parts; the real-mode solver stores only
// the real parts (double[n] per column).  These kernels are the complex ones
// above restricted to those real parts: the products they skip are the
// exact zeros, so every value equals what the complex kernels give.
// ---------------------------------------------------------------------------
#define ED_GROUP_R 16

struct ColPtrsR {
  const double* p[128];
};

static ColPtrsR make_cols_r(const double* const* cols, int nv) {
  ColPtrsR c;
  for (int i = 0; i < 128; ++i) c.p[i] = nullptr;
  for (int i = 0; i < nv && i < 128; ++i) c.p[i] = cols[i];
  return c;
}

// ---------------------------------------------------------------------------
// Float-pair products.  GB300 issues FP64 FMA at about 2 per clock per SM and
// FP32 FMA many times faster, and the restart combination V Y (16 x 8 FMAs
// per basis entry) is bound by the FP64 unit.  k_restart_pair keeps storage
// and the final sums in FP64 but forms the products on the FP32 units: each
// FP64 value v is read as a float pair hi + lo (integer operations on its
// bits: hi = the leading 24 significand bits, lo = the next 23 rounded,
// |v - hi - lo| <= 2^-47 |v|), products are formed exactly to first order
// (hi*hi exactly with an FMA, the three other terms added) and each thread
// sums them in a float pair with an error-free two-sum (Knuth's TwoSum).  The
// error of a product is below 2^-45 of |v y|; FP64 FMA over the 16 terms of
// an output is bounded by 16 x 2^-53 of the same sum, so the two agree to
// about 2^-45 relative.  Entries below 2^-126 in magnitude count as zero
// (below 2^-103 they lose lo); entries of 2^128 or more and non-finite ones
// give NaN.  For the Gram-Schmidt dots (one product per basis entry, so one
// split per product) the same arithmetic measured slower than FP64 FMA
// (6.9 against 5.5 ms at N=30), alone and split with FP64 columns, so those
// stay FP64.
// ---------------------------------------------------------------------------

// out_c = sum_i V_i Y[i][c] for 8 outputs per launch in float-pair products
// (Yp: the group's m x 8 coefficients as float pairs).  Measured at N=30:
// 14.9 ms per group against 32 ms in FP64 FMA, 22 ms with half the outputs
// in exact integers, and 21.7 ms with three of eight in FP64 beside five in
// pairs (the FP64 instructions do not overlap the FP32 work here).
__global__ void __launch_bounds__(256) k_restart_pair(const ColPtrsR cp, int m, const float2* __restrict__ Yp, int c0,
                                                      int nc, const ColPtrs outp, int64_t n) {
  __shared__ float2 shY[128 * 8];
  for (int k = threadIdx.x; k < m * 8; k += blockDim.x) shY[k] = Yp[k];
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    float s[8], c[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) s[k] = c[k] = 0.0f;
    for (int i = 0; i < m; ++i) {
      const float2 v = ed_pair(cp.p[i][r]);
#pragma unroll
      for (int k = 0; k < 8; ++k) ed_pair_mac(v, shY[i * 8 + k], s[k], c[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < nc) ((double*)outp.p[c0 + k])[r] = ed_pair_value(s[k], c[k]);
  }
}

// partial[item * nblk + blk]: items v0..v0+ng-1 = V_i^T w; item v0+ng = ||w||^2
// (with_norm).  LOCAL: first w <- w - a vj - b vjm1 (vjm1 may be null),
// written back.
template <int G, bool LOCAL>
__global__ void __launch_bounds__(ED_RED_THREADS) k_multidot_r(const ColPtrsR cp, int v0, int ng, double* __restrict__ w,
                                                               int64_t n, const double* __restrict__ vj, double a,
                                                               const double* __restrict__ vjm1, double b, int with_norm,
                                                               double* __restrict__ partial, int nblk) {
  double acc[G + 1];
#pragma unroll
  for (int k = 0; k <= G; ++k) acc[k] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double wv = w[r];
    if (LOCAL) {
      wv = fma(-a, vj[r], wv);
      if (vjm1) wv = fma(-b, vjm1[r], wv);
      w[r] = wv;
    }
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (g < ng) acc[g] = fma(cp.p[v0 + g][r], wv, acc[g]);
    if (with_norm) acc[G] = fma(wv, wv, acc[G]);
  }
  __shared__ double sh[(G + 1) * 32];
  ed_block_reduce<G + 1>(acc, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (g < ng) partial[(size_t)(v0 + g) * nblk + blockIdx.x] = acc[g];
    if (with_norm) partial[(size_t)(v0 + ng) * nblk + blockIdx.x] = acc[G];
  }
}

// h_host[i] = V_i^T w (i < nv), *wnorm2_host = ||w||^2 (after the local step
// when vj is given: w <- w - a vj - b vjm1 first, in the same pass as the
// first group of dots).
int ed_multidot_r(ed_ctx* ctx, const double* const* cols, int nv, double* w, int64_t n, const double* vj, double a,
                  const double* vjm1, double b, double* h_host, double* wnorm2_host) {
  if (nv > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  const int nblk = red_blocks(ctx, n);
  const int items = nv + 1;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)items * nblk + items));
  ColPtrsR cp = make_cols_r(cols, nv);
  const int ngroups = std::max(1, (nv + ED_GROUP_R - 1) / ED_GROUP_R);
  for (int gidx = 0; gidx < ngroups; ++gidx) {
    const int v0 = gidx * ED_GROUP_R;
    const int ng = std::max(0, std::min(ED_GROUP_R, nv - v0));
    const int last = gidx == ngroups - 1 && wnorm2_host != nullptr;  // the norm costs one FP64 FMA per row
    if (gidx == 0 && vj)
      k_multidot_r<ED_GROUP_R, true><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, vj, a, vjm1, b, last,
                                                                              ctx->d_red, nblk);
    else
      k_multidot_r<ED_GROUP_R, false><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, nullptr, 0.0, nullptr,
                                                                               0.0, last, ctx->d_red, nblk);
    ED_CHECK_LAUNCH(ctx);
  }
  std::vector<double> out(items);
  ED_TRY(ed_finish_reduce(ctx, items, nblk, out.data()));
  for (int i = 0; i < nv; ++i) h_host[i] = out[i];
  if (wnorm2_host) *wnorm2_host = out[nv];
  return ED_OK;
}

// w <- w - sum_i V_i h_i; partial ||w||^2.  Two rows per thread, columns
// unrolled by four.
__global__ void __launch_bounds__(ED_RED_THREADS) k_update_r(const ColPtrsR cp, int nv, const double* __restrict__ h,
                                                             double* __restrict__ w, int64_t n,
                                                             double* __restrict__ partial, int with_max) {
  __shared__ double sh_h[128];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) sh_h[i] = h[i];
  __syncthreads();
  double acc[1] = {0.0};
  unsigned int amax = 0u;  // high word of max |w|
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r0 < n; r0 += 2 * stride) {
    const int64_t r1 = r0 + stride;
    const bool has1 = r1 < n;
    double w0 = w[r0];
    double w1 = has1 ? w[r1] : 0.0;
#pragma unroll 4
    for (int i = 0; i < nv; ++i) {
      const double* col = cp.p[i];
      const double c = sh_h[i];
      w0 = fma(-col[r0], c, w0);
      if (has1) w1 = fma(-col[r1], c, w1);
    }
    w[r0] = w0;
    acc[0] = fma(w0, w0, acc[0]);
    if (with_max) amax = ed_absmax_hi(amax, w0);
    if (has1) {
      w[r1] = w1;
      acc[0] = fma(w1, w1, acc[0]);
      if (with_max) amax = ed_absmax_hi(amax, w1);
    }
  }
  __shared__ double shr[32];
  ed_block_reduce<1>(acc, shr);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
  if (with_max) {
    __syncthreads();  // shr reused
    double am = ed_absmax_hi_value(amax);
    ed_block_max(am, shr);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = am;
  }
}


template <int MAXM>
struct UpdLimbs;
template <int MAXM>
__global__ void k_update_fx(const ColPtrsR cp, int nv, const __grid_constant__ UpdLimbs<MAXM> H,
                            double* __restrict__ w, int64_t n, double* __restrict__ partial, int with_max);
template <int MAXM>
static int update_fx_launch(ed_ctx* ctx, const ColPtrsR& cp, int nv, const double* h_host, double* w, int64_t n,
                            int nblk, int with_max);

int ed_update_r(ed_ctx* ctx, const double* const* cols, int nv, const double* h_host, double* w, int64_t n,
                double* wnorm2_host, double* wmax_host, int arith) {
  if (nv > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  const bool fx = arith == ED_RESTART_FIXED && nv <= 32;
  int nblk = red_blocks(ctx, n);
  if (fx) {  // one full wave of the register-heavier integer kernel
    int per_sm = 0;
    if (nv <= 16) ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_update_fx<16>, ED_RED_THREADS, 0));
    else ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_update_fx<32>, ED_RED_THREADS, 0));
    const int64_t b = (n + ED_RED_THREADS - 1) / ED_RED_THREADS;
    nblk = (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)ctx->num_sms * std::max(1, per_sm)));
  }
  const int items = wmax_host ? 2 : 1;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)items * nblk + 4 + 128));
  double* h_dev = ctx->d_red + (size_t)items * nblk + 2;
  ED_CUDA(cudaMemcpyAsync(h_dev, h_host, sizeof(double) * nv, cudaMemcpyHostToDevice, ctx->stream));
  ColPtrsR cp = make_cols_r(cols, nv);
  int rc = ED_ENOTSUP;
  if (fx)
    rc = nv <= 16 ? update_fx_launch<16>(ctx, cp, nv, h_host, w, n, nblk, wmax_host ? 1 : 0)
                  : update_fx_launch<32>(ctx, cp, nv, h_host, w, n, nblk, wmax_host ? 1 : 0);
  if (rc == ED_ENOTSUP) {
    k_update_r<<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, nv, h_dev, w, n, ctx->d_red, wmax_host ? 1 : 0);
    ED_CHECK_LAUNCH(ctx);
  } else {
    ED_TRY(rc);
  }
  double out[2] = {0.0, 0.0};
  ED_TRY(ed_finish_reduce(ctx, items, nblk, out, items - 1));
  if (wnorm2_host) *wnorm2_host = out[0];
  if (wmax_host) *wmax_host = out[1];
  return ED_OK;
}

__global__ void k_scale_copy_r(const double* __restrict__ src, double* __restrict__ dst, double s, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) dst[r] = src[r] * s;
}

int ed_scale_copy_r(ed_ctx* ctx, const double* src, double* dst, double s, int64_t n) {
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_scale_copy_r<<<g, 256, 0, ctx->stream>>>(src, dst, s, n);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

// out_c = sum_i V_i * Y[i*ldY + c] for real storage.  GB300 runs FP64 FMA
// at a small fraction of its other rates, and the combination is bound by it
// (16 x 8 FMAs per element: 32 ms at N=30).  So the eight outputs of a group
// are split between two arithmetic units that work side by side: columns
// 0..3 in FP64 FMA, columns 4..7 in exact integer arithmetic.  For those,
// every column is a unit vector and Y is orthogonal, so |v|, |Y| <= 1: both
// become 62-bit fixed point (v in registers, Y on the host), each product is
// exact in 128 bits (__mul64hi and the low word), each sum is exact (by
// Cauchy-Schwarz it stays below sqrt(m), far inside 128 bits) and each output
// is rounded once.  Measured at N=30: 23 ms against 32 ms for all-FP64 and
// 32 ms for all-integer.  A non-finite input makes its row's integer
// outputs NaN, as the FP64 ones become.
__device__ __forceinline__ long long ed_fx62(double v, bool& bad) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((bits >> 52) & 0x7FF);
  if (e == 0x7FF) { bad = true; return 0; }
  if (e == 0) return 0;  // |v| < 2^-1022
  const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = e - 1013;  // v * 2^62 = mant * 2^(e - 1023 - 52 + 62)
  unsigned long long a;
  if (sh >= 0) a = mant << sh;  // |v| <= 1: sh <= 10, a <= 2^62
  else if (sh > -63) a = (mant + (1ull << (-sh - 1))) >> (-sh);
  else a = 0;
  return (bits >> 63) ? -(long long)a : (long long)a;
}

// NF outputs of a group in FP64 and the next NI in integers (NF + NI <= 8).
// A full group of eight takes 4 + 4, which keeps both units busy (3 + 5 and
// 4 + 4 measured the same; 2 + 6 and fewer FP64 outputs were slower).  A
// partial last group computes only the outputs it stores: one or two in FP64
// alone (an integer output of its own would pay the conversion of every input
// for one product), three or more split as evenly as the FP64 side allows.
template <int NF, int NI>
__global__ void __launch_bounds__(256) k_restart_mix(const ColPtrsR cp, int m, const double* __restrict__ Yd,
                                                     const long long* __restrict__ Yq, int c0,
                                                     const ColPtrs outp, int64_t n) {
  static_assert(NF >= 1 && NI >= 0 && NF + NI <= 8, "group of at most eight outputs");
  __shared__ double shY[128 * 8];     // m x 8 coefficients of this group (FP64 columns)
  __shared__ long long shQ[128 * 8];  // the same, 62-bit fixed point (integer columns)
  for (int k = threadIdx.x; k < m * 8; k += blockDim.x) {
    shY[k] = Yd[k];
    shQ[k] = Yq[k];
  }
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double a[NF];
    unsigned long long lo[NI > 0 ? NI : 1];
    long long hi[NI > 0 ? NI : 1];
#pragma unroll
    for (int c = 0; c < NF; ++c) a[c] = 0.0;
#pragma unroll
    for (int c = 0; c < NI; ++c) { lo[c] = 0ull; hi[c] = 0ll; }
    bool bad = false;
    for (int i = 0; i < m; ++i) {
      const double vd = cp.p[i][r];
#pragma unroll
      for (int c = 0; c < NF; ++c) a[c] = fma(vd, shY[i * 8 + c], a[c]);
      if (NI > 0) {
        const long long v = ed_fx62(vd, bad);
#pragma unroll
        for (int c = 0; c < NI; ++c) {
          const long long y = shQ[i * 8 + NF + c];
          const unsigned long long pl = (unsigned long long)v * (unsigned long long)y;
          const long long ph = __mul64hi(v, y);
          const unsigned long long s = lo[c] + pl;
          hi[c] += ph + (s < pl ? 1 : 0);
          lo[c] = s;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NF; ++c) ((double*)outp.p[c0 + c])[r] = a[c];
#pragma unroll
    for (int c = 0; c < NI; ++c) {
      // (hi * 2^64 + lo) * 2^-124
      double d = fma((double)hi[c], 0x1p-60, (double)lo[c] * 0x1p-124);
      if (bad) d = __longlong_as_double(0x7FF8000000000000ll);
      ((double*)outp.p[c0 + NF + c])[r] = d;
    }
  }
}

// One group of nc outputs (1..8) with the split above.
static int restart_mix_launch(ed_ctx* ctx, const ColPtrsR& cp, int m, const double* dYd, const long long* dYq, int c0,
                              int nc, const ColPtrs& op, int64_t n) {
  auto go = [&](auto kern) -> int {
    int per_sm = 0;
    ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0));
    if (per_sm < 1) per_sm = 1;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * per_sm));
    kern<<<g, 256, 0, ctx->stream>>>(cp, m, dYd, dYq, c0, op, n);
    ED_CHECK_LAUNCH(ctx);
    return ED_OK;
  };
  switch (nc) {
    case 1: return go(k_restart_mix<1, 0>);
    case 2: return go(k_restart_mix<2, 0>);
    case 3: return go(k_restart_mix<2, 1>);
    case 4: return go(k_restart_mix<2, 2>);
    case 5: return go(k_restart_mix<3, 2>);
    case 6: return go(k_restart_mix<3, 3>);
    case 7: return go(k_restart_mix<4, 3>);
    case 8: return go(k_restart_mix<4, 4>);
    default: return ed_fail(ED_EINVAL, "restart group of " + std::to_string(nc) + " outputs");
  }
}

// ---------------------------------------------------------------------------
// Restart combination on the integer units (ED_RESTART_FIXED).  Row r of
// output c is sum_i V_i[r] Y[i][c].  Each row's m entries are put in 56-bit
// fixed point against the row's largest exponent E (q = round(v 2^(1078 - E)),
// |q| <= 2^56), each coefficient column against its own (y = round(Y 2^(56 -
// F_c))), and both are split into 28-bit limbs, q = qh 2^28 + ql with
// ql in [0, 2^28).  The products are then exact sums of four 32 x 32 -> 64
// bit multiply-adds (mad.wide.s32, full rate on the integer pipe, against
// 1/64 rate for FP64 on this part); with m <= 32 none of the three partial
// sums can overflow 64 bits.  The exact 118-bit row sum is rounded once to
// FP64.  Error: half a unit of each fixed-point input, below 2^-51 of
// max_i |V_i[r]| * max_i |Y[i][c]| per output (an FP64 FMA chain over 16
// terms is bounded by 2^-49 of the same product).
// ---------------------------------------------------------------------------
template <int MAXM>
struct RsLimbs {
  int yh[MAXM * 8];  // [i][c]
  int yl[MAXM * 8];
  int z[8];  // output c = T 2^(E - 1078 + z[c])
};

__device__ __forceinline__ long long ed_mad_wide(int a, int b, long long c) {
  long long d;
  asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
  return d;
}

// round(v 2^(1078 - E)) for a row whose largest biased exponent is E
// (|result| <= 2^56); 0 for zeros and subnormals.
__device__ __forceinline__ long long ed_fx56_row(double v, int E) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0;
  const unsigned long long mant = (unsigned long long)(b & 0xFFFFFFFFFFFFFll) | 0x10000000000000ull;
  const int sh = e - E + 3;  // <= 3
  unsigned long long q;
  if (sh >= 0) q = mant << sh;
  else if (sh > -60) q = (mant + (1ull << (-sh - 1))) >> (-sh);
  else q = 0ull;
  return b < 0 ? -(long long)q : (long long)q;
}

template <int MAXM>
__global__ void __launch_bounds__(256, 2) k_restart_fx(const ColPtrsR cp, int m, int c0, int nc,
                                                       const __grid_constant__ RsLimbs<MAXM> Y, const ColPtrs outp,
                                                       int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double v[MAXM];
    int E = 0;
#pragma unroll
    for (int i = 0; i < MAXM; ++i) {
      v[i] = i < m ? cp.p[i][r] : 0.0;
      E = max(E, (int)((__double_as_longlong(v[i]) >> 52) & 0x7FF));
    }
    long long s1[8], s2[8], s3[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) s1[c] = s2[c] = s3[c] = 0ll;
#pragma unroll
    for (int i = 0; i < MAXM; ++i) {
      if (i < m) {
        const long long q = ed_fx56_row(v[i], E);
        const int qh = (int)(q >> 28), ql = (int)(q & 0xFFFFFFFll);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          s1[c] = ed_mad_wide(qh, Y.yh[i * 8 + c], s1[c]);
          s2[c] = ed_mad_wide(qh, Y.yl[i * 8 + c], s2[c]);
          s2[c] = ed_mad_wide(ql, Y.yh[i * 8 + c], s2[c]);
          s3[c] = ed_mad_wide(ql, Y.yl[i * 8 + c], s3[c]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (c < nc) {
        // T = s1 2^56 + s2 2^28 + s3 as a signed 128-bit (hi, lo)
        unsigned long long lo = (unsigned long long)s3[c];
        long long hi = s3[c] >> 63;
        unsigned long long a = (unsigned long long)s2[c] << 28, x = lo + a;
        hi += (s2[c] >> 36) + (x < lo ? 1ll : 0ll);
        lo = x;
        a = (unsigned long long)s1[c] << 56;
        x = lo + a;
        hi += (s1[c] >> 8) + (x < lo ? 1ll : 0ll);
        lo = x;
        double d = ed_fx128_to_double(hi, lo, E - 1078 + Y.z[c]);
        if (E == 0x7FF) d = __longlong_as_double(0x7FF8000000000000ll);
        ((double*)outp.p[c0 + c])[r] = d;
      }
    }
  }
}

template <int MAXM>
static int restart_fx_launch(ed_ctx* ctx, const ColPtrsR& cp, int m, const double* Y, int ldY, int l,
                             const ColPtrs& op, int64_t n) {
  int per_sm = 0;
  ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_restart_fx<MAXM>, 256, 0));
  if (per_sm < 1) per_sm = 1;
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * per_sm));
  for (int g0 = 0; g0 < l; g0 += 8) {
    const int nc = std::min(8, l - g0);
    RsLimbs<MAXM> P;
    std::memset(&P, 0, sizeof(P));
    for (int c = 0; c < nc; ++c) {
      double mx = 0.0;
      for (int i = 0; i < m; ++i) {
        const double y = Y[(size_t)i * ldY + g0 + c];
        if (!std::isfinite(y)) return ed_fail(ED_EINVAL, "non-finite restart coefficient");
        mx = std::max(mx, std::fabs(y));
      }
      int F = 0;
      if (mx > 0.0) std::frexp(mx, &F);  // mx < 2^F
      P.z[c] = F - 56;
      for (int i = 0; i < m; ++i) {
        const long long y = std::llround(std::ldexp(Y[(size_t)i * ldY + g0 + c], 56 - F));  // |y| <= 2^56
        P.yh[i * 8 + c] = (int)(y >> 28);
        P.yl[i * 8 + c] = (int)(y & 0xFFFFFFFll);
      }
    }
    k_restart_fx<MAXM><<<g, 256, 0, ctx->stream>>>(cp, m, g0, nc, P, op, n);
    ED_CHECK_LAUNCH(ctx);
  }
  return ED_OK;
}

// w <- w - sum_i V_i h_i on the integer units (ED_RESTART_FIXED): row r's
// entries V_i[r] in 56-bit fixed point against the row's largest exponent,
// h in 56-bit fixed point against max|h_i|, exact products of 28-bit limbs,
// the row's sum rounded once to FP64 and subtracted (one FP64 add per row
// instead of nv FP64 FMAs).  Partial ||w||^2 and the high word of max |w|
// as k_update_r.
template <int MAXM>
struct UpdLimbs {
  int hh[MAXM];
  int hl[MAXM];
  int z;  // sum = T 2^(E - 1078 + z)
};

template <int MAXM>
__global__ void __launch_bounds__(ED_RED_THREADS) k_update_fx(const ColPtrsR cp, int nv,
                                                              const __grid_constant__ UpdLimbs<MAXM> H,
                                                              double* __restrict__ w, int64_t n,
                                                              double* __restrict__ partial, int with_max) {
  double acc[1] = {0.0};
  unsigned int amax = 0u;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double v[MAXM];
    int E = 0;
#pragma unroll
    for (int i = 0; i < MAXM; ++i) {
      v[i] = i < nv ? cp.p[i][r] : 0.0;
      E = max(E, (int)((__double_as_longlong(v[i]) >> 52) & 0x7FF));
    }
    long long s1 = 0, s2 = 0, s3 = 0;
#pragma unroll
    for (int i = 0; i < MAXM; ++i) {
      if (i < nv) {
        const long long q = ed_fx56_row(v[i], E);
        const int qh = (int)(q >> 28), ql = (int)(q & 0xFFFFFFFll);
        s1 = ed_mad_wide(qh, H.hh[i], s1);
        s2 = ed_mad_wide(qh, H.hl[i], s2);
        s2 = ed_mad_wide(ql, H.hh[i], s2);
        s3 = ed_mad_wide(ql, H.hl[i], s3);
      }
    }
    unsigned long long lo = (unsigned long long)s3;
    long long hi = s3 >> 63;
    unsigned long long a = (unsigned long long)s2 << 28, x = lo + a;
    hi += (s2 >> 36) + (x < lo ? 1ll : 0ll);
    lo = x;
    a = (unsigned long long)s1 << 56;
    x = lo + a;
    hi += (s1 >> 8) + (x < lo ? 1ll : 0ll);
    lo = x;
    double d = ed_fx128_to_double(hi, lo, E - 1078 + H.z);
    if (E == 0x7FF) d = __longlong_as_double(0x7FF8000000000000ll);
    const double wv = w[r] - d;
    w[r] = wv;
    acc[0] = fma(wv, wv, acc[0]);
    if (with_max) amax = ed_absmax_hi(amax, wv);
  }
  __shared__ double shr[32];
  ed_block_reduce<1>(acc, shr);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
  if (with_max) {
    __syncthreads();  // shr reused
    double am = ed_absmax_hi_value(amax);
    ed_block_max(am, shr);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = am;
  }
}

template <int MAXM>
static int update_fx_launch(ed_ctx* ctx, const ColPtrsR& cp, int nv, const double* h_host, double* w, int64_t n,
                            int nblk, int with_max) {
  UpdLimbs<MAXM> P;
  std::memset(&P, 0, sizeof(P));
  double mx = 0.0;
  for (int i = 0; i < nv; ++i) {
    if (!std::isfinite(h_host[i])) return ED_ENOTSUP;  // the FP64 form propagates it
    mx = std::max(mx, std::fabs(h_host[i]));
  }
  int F = 0;
  if (mx > 0.0) std::frexp(mx, &F);  // mx < 2^F
  P.z = F - 56;
  for (int i = 0; i < nv; ++i) {
    const long long y = std::llround(std::ldexp(h_host[i], 56 - F));  // |y| <= 2^56
    P.hh[i] = (int)(y >> 28);
    P.hl[i] = (int)(y & 0xFFFFFFFll);
  }
  k_update_fx<MAXM><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, nv, P, w, n, ctx->d_red, with_max);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

int ed_restart_combine_r(ed_ctx* ctx, const double* const* cols, int m, const double* Y, int ldY, int l,
                         double* const* out, int64_t n, int arith) {
  if (m > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  if (arith == ED_RESTART_EXACT) return ed_restart_combine_tc(ctx, cols, m, Y, ldY, l, out, n);
  const bool pair = arith == ED_RESTART_PAIR;
  ColPtrsR cp = make_cols_r(cols, m);
  ColPtrs op;
  for (int i = 0; i < 128; ++i) op.p[i] = nullptr;
  for (int i = 0; i < l && i < 128; ++i) op.p[i] = (const double2*)out[i];
  if (arith == ED_RESTART_FIXED && m <= 32) {
    if (m <= 16) return restart_fx_launch<16>(ctx, cp, m, Y, ldY, l, op, n);
    return restart_fx_launch<32>(ctx, cp, m, Y, ldY, l, op, n);
  }
  const int ngroups = (l + 7) / 8;
  const size_t per = (size_t)m * 8;
  if (pair) {
    // coefficients per group of 8 outputs, [group][i][8], as float pairs
    std::vector<float2> yp(ngroups * per, make_float2(0.0f, 0.0f));
    for (int gi = 0; gi < ngroups; ++gi)
      for (int i = 0; i < m; ++i)
        for (int c = 0; c < 8 && gi * 8 + c < l; ++c) yp[(gi * m + i) * 8 + c] = ed_host_pair(Y[(size_t)i * ldY + gi * 8 + c]);
    ED_TRY(ed_ensure_reduce(ctx, ngroups * per + 16));
    float2* dYp = (float2*)ctx->d_red;
    ED_CUDA(cudaMemcpyAsync(dYp, yp.data(), sizeof(float2) * yp.size(), cudaMemcpyHostToDevice, ctx->stream));
    int per_sm = 0;
    ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_restart_pair, 256, 0));
    if (per_sm < 1) per_sm = 1;
    int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * per_sm));
    for (int gi = 0; gi < ngroups; ++gi) {
      k_restart_pair<<<g, 256, 0, ctx->stream>>>(cp, m, dYp + gi * per, gi * 8, std::min(8, l - gi * 8), op, n);
      ED_CHECK_LAUNCH(ctx);
    }
    // the host coefficients must outlive the copies
    ED_CUDA(cudaStreamSynchronize(ctx->stream));
    return ED_OK;
  }
  // coefficients per group of 8 outputs, [group][i][8]: FP64 and 62-bit fixed point
  std::vector<double> yd(ngroups * per, 0.0);
  std::vector<long long> yq(ngroups * per, 0);
  for (int gi = 0; gi < ngroups; ++gi)
    for (int i = 0; i < m; ++i)
      for (int c = 0; c < 8; ++c) {
        const int col = gi * 8 + c;
        if (col >= l) continue;
        const double y = Y[(size_t)i * ldY + col];
        yd[(gi * m + i) * 8 + c] = y;
        yq[(gi * m + i) * 8 + c] = std::llround(std::ldexp(y, 62));
      }
  ED_TRY(ed_ensure_reduce(ctx, 2 * ngroups * per + 16));
  double* dYd = ctx->d_red;
  long long* dYq = (long long*)(ctx->d_red + ngroups * per);
  ED_CUDA(cudaMemcpyAsync(dYd, yd.data(), sizeof(double) * yd.size(), cudaMemcpyHostToDevice, ctx->stream));
  ED_CUDA(cudaMemcpyAsync(dYq, yq.data(), sizeof(long long) * yq.size(), cudaMemcpyHostToDevice, ctx->stream));
  for (int gi = 0; gi < ngroups; ++gi)
    ED_TRY(restart_mix_launch(ctx, cp, m, dYd + gi * per, dYq + gi * per, gi * 8, std::min(8, l - gi * 8), op, n));
  // the host coefficients must outlive the copies
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  return ED_OK;
}

__global__ void __launch_bounds__(ED_RED_THREADS) k_residual_r(const double* __restrict__ hx, const double* __restrict__ x,
                                                               double theta, int64_t n, double* __restrict__ partial,
                                                               int nblk) {
  double acc[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const double d = fma(-theta, x[r], hx[r]);
    acc[0] = fma(d, d, acc[0]);
    acc[1] = fma(x[r], x[r], acc[1]);
  }
  __shared__ double sh[64];
  ed_block_reduce<2>(acc, sh);
  if (threadIdx.x == 0) { partial[blockIdx.x] = acc[0]; partial[nblk + blockIdx.x] = acc[1]; }
}

int ed_residual_norm2_r(ed_ctx* ctx, const double* hx, const double* x, double theta, int64_t n, double* r2_host,
                        double* x2_host) {
  const int nblk = red_blocks(ctx, n);
  ED_TRY(ed_ensure_reduce(ctx, (size_t)2 * nblk + 2));
  k_residual_r<<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(hx, x, theta, n, ctx->d_red, nblk);
  ED_CHECK_LAUNCH(ctx);
  double out[2] = {0.0, 0.0};
  ED_TRY(ed_finish_reduce(ctx, 2, nblk, out));
  *r2_host = out[0];
  *x2_host = out[1];
  return ED_OK;
}

// Real parts of the seeded start vector (the same values k_start_vector
// writes into the real parts).
__global__ void k_start_vector_r(uint64_t seed, int64_t n, double* __restrict__ v) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const uint64_t base = seed * 0xD1B54A32D192ED03ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t h1 = ed_splitmix64(base + 2 * (uint64_t)i);
    const double u1 = (double)(h1 >> 11) * (1.0 / 9007199254740992.0);
    v[i] = 2.0 * u1 - 1.0;
  }
}

int ed_start_vector_r(ed_ctx* ctx, uint64_t seed, int64_t n, double* v) {
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_start_vector_r<<<g, 256, 0, ctx->stream>>>(seed, n, v);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

__global__ void k_real_to_complex(const double* __restrict__ src, double2* __restrict__ dst, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    dst[i] = make_double2(src[i], 0.0);
}

__global__ void k_complex_to_real(const double2* __restrict__ src, double* __restrict__ dst, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i].x;
}

int ed_real_to_complex(ed_ctx* ctx, const double* src, double2* dst, int64_t n) {
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_real_to_complex<<<g, 256, 0, ctx->stream>>>(src, dst, n);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

int ed_complex_to_real(ed_ctx* ctx, const double2* src, double* dst, int64_t n) {
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_complex_to_real<<<g, 256, 0, ctx->stream>>>(src, dst, n);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}
