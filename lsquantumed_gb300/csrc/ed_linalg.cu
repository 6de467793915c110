// Vector kernels of the Krylov-Schur solver (complex128, device-resident).
// Reductions are two-stage with a fixed block count and a fixed tree order,
// so every result is bit-reproducible run to run.
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>

#define ED_RED_THREADS 256
#define ED_GROUP 8

struct ColPtrs {
  const double2* p[128];
};

static int red_blocks(ed_ctx* ctx, int64_t n) {
  int64_t b = (n + ED_RED_THREADS - 1) / ED_RED_THREADS;
  int64_t cap = (int64_t)ctx->num_sms * 2;
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

// Block reduction of NV doubles; thread 0 of the block ends with the sums in out[].
template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], double* sh /* [NV][32] */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) sh[k * 32 + wid] = a;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double a = lane < nw ? sh[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      v[k] = a;
    }
  }
}

// partial[item * nblk + blk]
template <int G>
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
        acc[2 * g] = fma(v.x, wv.x, fma(v.y, wv.y, acc[2 * g]));
        acc[2 * g + 1] = fma(v.x, wv.y, fma(-v.y, wv.x, acc[2 * g + 1]));
      }
    }
    if (with_norm) acc[2 * G] = fma(wv.x, wv.x, fma(wv.y, wv.y, acc[2 * G]));
  }
  __shared__ double sh[(2 * G + 1) * 32];
  block_reduce<2 * G + 1>(acc, sh);
  if (threadIdx.x == 0) {
    for (int g = 0; g < ng; ++g) {
      partial[(size_t)(2 * (v0 + g)) * nblk + blockIdx.x] = acc[2 * g];
      partial[(size_t)(2 * (v0 + g) + 1) * nblk + blockIdx.x] = acc[2 * g + 1];
    }
    if (with_norm) partial[(size_t)(2 * (v0 + ng)) * nblk + blockIdx.x] = acc[2 * G];
  }
}

// Second stage: out[item] = sum_b partial[item*nblk + b] (fixed order).
__global__ void k_reduce_items(const double* __restrict__ partial, int nblk, double* __restrict__ out) {
  __shared__ double sh[256];
  const int item = blockIdx.x;
  double a = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) a += partial[(size_t)item * nblk + b];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[item] = sh[0];
}

static int finish_reduce(ed_ctx* ctx, int items, int nblk, double* host_out) {
  double* out_dev = ctx->d_red + (size_t)items * nblk;
  k_reduce_items<<<items, 256, 0, ctx->stream>>>(ctx->d_red, nblk, out_dev);
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
                double* wnorm2_host) {
  if (nv > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  const int nblk = red_blocks(ctx, n);
  const int items = 2 * nv + 1;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)items * nblk + items));
  ColPtrs cp = make_cols(cols, nv);
  int with_norm_done = 0;
  for (int v0 = 0; v0 < nv || !with_norm_done; v0 += ED_GROUP) {
    int ng = std::max(0, std::min(ED_GROUP, nv - v0));
    int last = (v0 + ED_GROUP >= nv);
    k_multidot<ED_GROUP><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, last, ctx->d_red, nblk);
    ED_CHECK_LAUNCH(ctx);
    if (last) with_norm_done = 1;
  }
  std::vector<double> out(items);
  ED_TRY(finish_reduce(ctx, items, nblk, out.data()));
  for (int i = 0; i < nv; ++i) { h_host[i].x = out[2 * i]; h_host[i].y = out[2 * i + 1]; }
  if (wnorm2_host) *wnorm2_host = out[2 * nv];
  return ED_OK;
}

// Local Lanczos projection fused with the first group of the full CGS dot
// products: w <- w - a v_j - b v_{j-1} (written back when `local` is set),
// then partial[i] = V_{v0+i}^H w and ||w||^2.
template <int G>
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
      wv.x = fma(-a.x, p.x, fma(a.y, p.y, wv.x));
      wv.y = fma(-a.x, p.y, fma(-a.y, p.x, wv.y));
      if (vjm1) {
        const double2 q = vjm1[r];
        wv.x = fma(-b, q.x, wv.x);
        wv.y = fma(-b, q.y, wv.y);
      }
      w[r] = wv;
    }
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g < ng) {
        const double2 v = cp.p[v0 + g][r];
        acc[2 * g] = fma(v.x, wv.x, fma(v.y, wv.y, acc[2 * g]));
        acc[2 * g + 1] = fma(v.x, wv.y, fma(-v.y, wv.x, acc[2 * g + 1]));
      }
    }
    if (with_norm) acc[2 * G] = fma(wv.x, wv.x, fma(wv.y, wv.y, acc[2 * G]));
  }
  __shared__ double sh[(2 * G + 1) * 32];
  block_reduce<2 * G + 1>(acc, sh);
  if (threadIdx.x == 0) {
    for (int g = 0; g < ng; ++g) {
      partial[(size_t)(2 * (v0 + g)) * nblk + blockIdx.x] = acc[2 * g];
      partial[(size_t)(2 * (v0 + g) + 1) * nblk + blockIdx.x] = acc[2 * g + 1];
    }
    if (with_norm) partial[(size_t)(2 * (v0 + ng)) * nblk + blockIdx.x] = acc[2 * G];
  }
}

int ed_local_multidot(ed_ctx* ctx, const double2* const* cols, int nv, double2* w, int64_t n, const double2* vj,
                      double2 a, const double2* vjm1, double b, double2* h_host, double* wnorm2_host) {
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
    k_local_multidot<ED_GROUP><<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, v0, ng, w, n, gidx == 0, vj, a, vjm1, b,
                                                                         last, ctx->d_red, nblk);
    ED_CHECK_LAUNCH(ctx);
  }
  std::vector<double> out(items);
  ED_TRY(finish_reduce(ctx, items, nblk, out.data()));
  for (int i = 0; i < nv; ++i) { h_host[i].x = out[2 * i]; h_host[i].y = out[2 * i + 1]; }
  if (wnorm2_host) *wnorm2_host = out[2 * nv];
  return ED_OK;
}

// w <- w - sum_i V_i h_i ; partial ||w||^2
__global__ void __launch_bounds__(ED_RED_THREADS) k_update(const ColPtrs cp, int nv, const double2* __restrict__ h,
                                                           double2* __restrict__ w, int64_t n, double* __restrict__ partial,
                                                           int nblk) {
  __shared__ double2 sh_h[128];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) sh_h[i] = h[i];
  __syncthreads();
  double acc[1] = {0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    double2 wv = w[r];
    for (int i = 0; i < nv; ++i) {
      const double2 v = cp.p[i][r];
      const double2 c = sh_h[i];
      wv.x = fma(-v.x, c.x, fma(v.y, c.y, wv.x));
      wv.y = fma(-v.x, c.y, fma(-v.y, c.x, wv.y));
    }
    w[r] = wv;
    acc[0] = fma(wv.x, wv.x, fma(wv.y, wv.y, acc[0]));
  }
  __shared__ double sh[32];
  block_reduce<1>(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
}

int ed_update(ed_ctx* ctx, const double2* const* cols, int nv, const double2* h_host, double2* w, int64_t n,
              double* wnorm2_host) {
  if (nv > 127) return ed_fail(ED_ENOTSUP, "at most 127 basis vectors");
  const int nblk = red_blocks(ctx, n);
  ED_TRY(ed_ensure_reduce(ctx, (size_t)nblk + 4 + 2 * 128));
  // h goes after the partials and the result slot, on a 16-byte boundary
  double2* h_dev = (double2*)(ctx->d_red + ((nblk + 2 + 1) & ~1));
  ED_CUDA(cudaMemcpyAsync(h_dev, h_host, sizeof(double2) * nv, cudaMemcpyHostToDevice, ctx->stream));
  ColPtrs cp = make_cols(cols, nv);
  k_update<<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(cp, nv, h_dev, w, n, ctx->d_red, nblk);
  ED_CHECK_LAUNCH(ctx);
  double out;
  ED_TRY(finish_reduce(ctx, 1, nblk, &out));
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
        ai[c] = fma(v.y, y, ai[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (c < nc) ((double2*)outp.p[c0 + c])[r] = make_double2(ar[c], ai[c]);
  }
}

int ed_restart_combine(ed_ctx* ctx, const double2* const* cols, int m, const double* Y, int ldY, int l,
                       double2* const* out, int64_t n) {
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
    k_restart<<<g, 256, smem, ctx->stream>>>(cp, m, dY, ldY, c0, nc, op, n);
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
  block_reduce<2>(acc, sh);
  if (threadIdx.x == 0) { partial[blockIdx.x] = acc[0]; partial[nblk + blockIdx.x] = acc[1]; }
}

int ed_residual_norm2(ed_ctx* ctx, const double2* hx, const double2* x, double theta, int64_t n, double* r2_host,
                      double* x2_host) {
  const int nblk = red_blocks(ctx, n);
  ED_TRY(ed_ensure_reduce(ctx, (size_t)2 * nblk + 2));
  k_residual<<<nblk, ED_RED_THREADS, 0, ctx->stream>>>(hx, x, theta, n, ctx->d_red, nblk);
  ED_CHECK_LAUNCH(ctx);
  double out[2];
  ED_TRY(finish_reduce(ctx, 2, nblk, out));
  *r2_host = out[0];
  *x2_host = out[1];
  return ED_OK;
}

// Deterministic start vector: re, im ~ U[-1, 1) from a counter hash (same
// bits as the CPU oracle's start vector).
__global__ void k_start_vector(uint64_t seed, int64_t n, double2* __restrict__ v) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const uint64_t base = seed * 0xD1B54A32D192ED03ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t h1 = ed_splitmix64(base + 2 * (uint64_t)i);
    const uint64_t h2 = ed_splitmix64(base + 2 * (uint64_t)i + 1);
    const double u1 = (double)(h1 >> 11) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);
    v[i] = make_double2(2.0 * u1 - 1.0, 2.0 * u2 - 1.0);
  }
}

int ed_start_vector(ed_ctx* ctx, uint64_t seed, int64_t n, double2* v) {
  int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  k_start_vector<<<g, 256, 0, ctx->stream>>>(seed, n, v);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}
