// Measurements: correlation expectation values (SzSz / SpSm / SmSp / SiSj,
// src/spinOperators/correlation.cpp:38-299) and DSF coefficients
// c_{i,n} = <v_n | S_i | psi0> (include/phys.tmpl_func.hpp:161-186 with
// Sqz / Sqp from include/spinOperators/spinOPft.tmpl_func.hpp).
//
// The reference builds a sparse operator matrix per (i, j) and runs MatMult +
// VecDot; here each pass over the basis evaluates a group of pairs at once,
// gathering psi at the rank of the flipped state.  The PETSc VecDot
// convention is kept: ExpectVal = sum_s psi_s * conj((O psi)_s).
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>

#define MEAS_G 8
#define MEAS_GR 16  // pairs per pass when psi is real

struct PairGroup {
  int n;
  int32_t i[MEAS_GR], j[MEAS_GR];
};

// Groups of up to G pairs per pass over the basis.  Ranks of flipped states
// come from the basis's two-table rank (T0 in shared memory, T1 through the
// read-only cache).  REAL: psi has zero imaginary parts (then every result is
// real and only real parts are accumulated; G = 16 pairs share one pass); a
// real psi normally takes k_expect_zz_r / k_expect_flip_r below, and this
// form only when their compact copy does not fit or psi is not finite.
template <int G, bool REAL>
__global__ void __launch_bounds__(256) k_expect(const uint32_t* __restrict__ states, const double2* __restrict__ psi,
                                                int64_t dim, const uint16_t* __restrict__ t0,
                                                const uint32_t* __restrict__ t1, int w0, int op, const PairGroup pg,
                                                double* __restrict__ partial, int nblk) {
  extern __shared__ uint16_t t0s[];
  for (int i = threadIdx.x; i < (1 << w0); i += blockDim.x) t0s[i] = t0[i];
  __syncthreads();
  constexpr int NA = REAL ? G : 2 * G;
  double acc[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) acc[k] = 0.0;
  const uint32_t low = (1u << w0) - 1u;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const uint32_t s = states[r];
    const double2 p = psi[r];
    const double w = REAL ? p.x * p.x : fma(p.x, p.x, p.y * p.y);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g < pg.n) {
        const int i = pg.i[g], j = pg.j[g];
        const uint32_t a = (s >> i) & 1u, b = (s >> j) & 1u;
        double cr = 0.0, ci = 0.0;
        // S^z_i S^z_j part: psi * conj(0.25 * (+-1) * psi)
        if (op == ED_OP_SZSZ || op == ED_OP_SISJ) cr += (a ^ b) ? -0.25 * w : 0.25 * w;
        if (op != ED_OP_SZSZ) {
          const double half = (op == ED_OP_SISJ) ? 0.5 : 1.0;
          if (i == j) {
            // S+S- = n_i (a = 1), S-S+ = 1 - n_i (a = 0)
            const bool on = (op == ED_OP_SPSM) ? (a == 1u) : (op == ED_OP_SMSP) ? (a == 0u) : true;
            if (on) cr += half * w;
          } else {
            const bool on = (op == ED_OP_SPSM) ? (a == 0u && b == 1u) : (op == ED_OP_SMSP) ? (a == 1u && b == 0u) : (a != b);
            if (on) {
              const uint32_t f = s ^ ((1u << i) | (1u << j));
              const uint32_t c = (uint32_t)t0s[f & low] + __ldg(&t1[f >> w0]);
              const double2 q = __ldg(&psi[c]);
              // psi_r * conj(psi_c)
              if (REAL) {
                cr += half * (p.x * q.x);
              } else {
                cr += half * fma(p.x, q.x, p.y * q.y);
                ci += half * fma(p.y, q.x, -p.x * q.y);
              }
            }
          }
        }
        if (REAL) {
          acc[g] += cr;
        } else {
          acc[2 * g] += cr;
          acc[2 * g + 1] += ci;
        }
      }
    }
  }
  __shared__ double sh[NA * 32];
  ed_block_reduce<NA>(acc, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NA; ++k) partial[(size_t)k * nblk + blockIdx.x] = acc[k];
  }
}

__global__ void k_sum_partials(const double* __restrict__ partial, int nblk, int items, double* __restrict__ out) {
  const int item = blockIdx.x;
  if (item >= items) return;
  __shared__ double sh[256];
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

template <int G, bool REAL>
static int expect_g(const ed_basis* b, int op, const double2* psi, const int32_t* pairs, int64_t np, double2* out) {
  ed_ctx* ctx = b->ctx;
  const int64_t dim = b->dim;
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((dim + 255) / 256, (int64_t)ctx->num_sms * 4));
  const int items = REAL ? G : 2 * G;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)items * nblk + items + 8));
  const size_t smem = sizeof(uint16_t) * ((size_t)1 << b->lin_w0);
  double* out_dev = ctx->d_red + (size_t)items * nblk;
  for (int64_t p0 = 0; p0 < np; p0 += G) {
    PairGroup pg;
    memset(&pg, 0, sizeof(pg));
    pg.n = (int)std::min<int64_t>(G, np - p0);
    for (int g = 0; g < pg.n; ++g) {
      pg.i[g] = pairs[2 * (p0 + g)];
      pg.j[g] = pairs[2 * (p0 + g) + 1];
    }
    k_expect<G, REAL><<<nblk, 256, smem, ctx->stream>>>(b->d_states, psi, dim, b->d_lin_t0, b->d_lin_t1, b->lin_w0, op,
                                                        pg, ctx->d_red, nblk);
    ED_CHECK_LAUNCH(ctx);
    k_sum_partials<<<items, 256, 0, ctx->stream>>>(ctx->d_red, nblk, items, out_dev);
    ED_CHECK_LAUNCH(ctx);
    ED_CUDA(cudaMemcpyAsync(ctx->h_red, out_dev, sizeof(double) * items, cudaMemcpyDeviceToHost, ctx->stream));
    ED_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int g = 0; g < pg.n; ++g) {
      out[p0 + g].x = REAL ? ctx->h_red[g] : ctx->h_red[2 * g];
      out[p0 + g].y = REAL ? 0.0 : ctx->h_red[2 * g + 1];
    }
  }
  return ED_OK;
}

// Real psi (the solver's eigenvectors) and any of the four operators; the
// all-pairs measurement.  For a real psi, <S+_i S-_j> = <S-_i S+_j> = F_ij,
// the flip sum below, for i != j.  The general kernel above spends
// about four FP64 operations per pair and row, and GB300 runs FP64 at a small
// fraction of its other rates: at N=30 that pass is FP64-bound.  Here two
// kernels share a pass of up to MEAS_GR pairs:
//  * k_expect_zz_r, the S^z S^z part 0.25 sum_r w_r sigma_i sigma_j with
//    w_r = psi_r^2 (FP64, as the general kernel forms it): each w_r becomes a
//    128-bit integer at the scale 2^(124 - e), sum_r w_r < 2^e, which holds
//    every w_r above 2^(e - 72) exactly; the sums T = sum_r w_r and, per pair,
//    A = sum over antiparallel rows of w_r (for i == j: over the rows with
//    spin i up, for S+S- and S-S+) are exact integer sums, and 0.25 (T - 2 A)
//    is rounded once at the end;
//  * k_expect_flip_r, the flip part (S+_i S-_j + S-_i S+_j) / 2: it pairs
//    every antiparallel row with its partner r' = rank(s ^ m) (an
//    involution), so it equals the sum over the rows with bit i set and bit j
//    clear of psi_r psi_r'.  Lane l of a warp serves pair l / 2: a ballot per
//    pair marks the contributing rows among the warp's 32, and the pair's two
//    lanes take alternate marked rows (state, psi and rank halves by
//    shuffle), four gathers in flight each.  A row and pair that contribute
//    nothing cost no FMA and no gather;
//  * psi is read as 8-byte real parts from a compact copy, and the next
//    chunk's rows are loaded while the current one is worked on;
//  * the row's own rank r = T0[s_lo] + T1[s_hi] gives both halves of the
//    flipped state's rank, so a flip inside the low bits needs no T1 load and
//    one inside the high bits no T0 lookup.
struct PairMasks {
  int n;
  uint32_t diag;         // bit g: pair g has i == j
  uint32_t m[MEAS_GR];   // (1 << i) | (1 << j)
  uint32_t bi[MEAS_GR];  // 1 << i
  uint32_t ml[MEAS_GR];  // m & (2^w0 - 1)
  uint32_t mh[MEAS_GR];  // m >> w0
};

// 128-bit integer accumulators (two 64-bit words, add with carry)
__device__ __forceinline__ void ed_add128(unsigned long long& lo, unsigned long long& hi, unsigned long long alo,
                                          unsigned long long ahi) {
  asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(alo), "l"(ahi));
}

// w >= 0 (finite) as the 128-bit integer round(w 2^S); exact when w's last
// bit is at or above 2^-S.  w < 2^(124 - S) keeps it below 2^124.
__device__ __forceinline__ void ed_fx128(double w, int S, unsigned long long& lo, unsigned long long& hi) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(w);
  const int E = (int)((bits >> 52) & 0x7FF);
  const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = E - 1075 + S;  // w 2^S = mant 2^sh
  lo = 0ull;
  hi = 0ull;
  if (E == 0) return;  // zero or below 2^-1022
  if (sh >= 64) {
    hi = mant << (sh - 64);
  } else if (sh > 0) {
    lo = mant << sh;
    hi = mant >> (64 - sh);
  } else if (sh == 0) {
    lo = mant;
  } else if (sh > -54) {
    lo = (mant + (1ull << (-sh - 1))) >> (-sh);
  }
}

// partial[(3 g) nblk + blk] and [(3 g + 1) nblk + blk]: lo and hi words of
// pair g's sum A over its antiparallel rows (i != j) or over the rows with
// spin i up (i == j); partial[(3 MEAS_GR) nblk + blk], [(3 MEAS_GR
// + 1) nblk + blk]: the block's T (int64 bits in the double array).
__global__ void __launch_bounds__(256, 2) k_expect_zz_r(const uint32_t* __restrict__ states,
                                                     const double* __restrict__ pr, int64_t dim, int S,
                                                     const PairMasks pm, double* __restrict__ partial, int nblk) {
  unsigned long long alo[MEAS_GR], ahi[MEAS_GR];
#pragma unroll
  for (int k = 0; k < MEAS_GR; ++k) { alo[k] = 0ull; ahi[k] = 0ull; }
  unsigned long long tlo = 0ull, thi = 0ull;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t s_n = 0u;
  double x_n = 0.0;
  if (r < dim) {
    s_n = states[r];
    x_n = pr[r];
  }
  for (; r < dim; r += stride) {
    const uint32_t s = s_n;
    const double x = x_n;
    if (r + stride < dim) {  // the next row, loaded while this one is worked on
      s_n = states[r + stride];
      x_n = pr[r + stride];
    }
    unsigned long long wlo, whi;
    ed_fx128(x * x, S, wlo, whi);
    ed_add128(tlo, thi, wlo, whi);
#pragma unroll
    for (int g = 0; g < MEAS_GR; ++g) {
      if (g < pm.n) {
        const uint32_t m = pm.m[g], bits = s & m;
        // i != j: antiparallel rows; i == j: rows with the spin up
        const bool hit = ((pm.diag >> g) & 1u) ? bits != 0u : (bits != 0u && bits != m);
        if (hit) ed_add128(alo[g], ahi[g], wlo, whi);
      }
    }
  }
  // block sums: warp shuffles with carries, then lane 0 of each warp in
  // shared memory, summed by thread 0 in a fixed order
  __shared__ unsigned long long shz[(MEAS_GR + 1) * 2 * 8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k <= MEAS_GR; ++k) {
    unsigned long long lo = k < MEAS_GR ? alo[k] : tlo, hi = k < MEAS_GR ? ahi[k] : thi;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long olo = __shfl_down_sync(0xffffffffu, lo, o), ohi = __shfl_down_sync(0xffffffffu, hi, o);
      ed_add128(lo, hi, olo, ohi);
    }
    if (lane == 0) {
      shz[(k * 8 + wid) * 2] = lo;
      shz[(k * 8 + wid) * 2 + 1] = hi;
    }
  }
  __syncthreads();
  if (threadIdx.x <= MEAS_GR) {
    const int k = threadIdx.x;
    unsigned long long lo = 0ull, hi = 0ull;
    for (int w = 0; w < nw; ++w) ed_add128(lo, hi, shz[(k * 8 + w) * 2], shz[(k * 8 + w) * 2 + 1]);
    partial[(size_t)(3 * k) * nblk + blockIdx.x] = __longlong_as_double((long long)lo);
    partial[(size_t)(3 * k + 1) * nblk + blockIdx.x] = __longlong_as_double((long long)hi);
  }
}

// partial[(3 g + 2) nblk + blk]: flip sum of pair g (FP64).
#define FL_U 4
__global__ void __launch_bounds__(256, 3) k_expect_flip_r(const uint32_t* __restrict__ states,
                                                       const double* __restrict__ pr, int64_t dim,
                                                       const uint16_t* __restrict__ t0,
                                                       const uint32_t* __restrict__ t1, int w0, const PairMasks pm,
                                                       double* __restrict__ partial, int nblk) {
  extern __shared__ uint16_t t0s[];
  for (int i = threadIdx.x; i < (1 << w0); i += blockDim.x) t0s[i] = t0[i];
  __syncthreads();
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int gl = lane >> 1, par = lane & 1;  // this lane's pair and its turn
  const bool gl_on = gl < pm.n && !((pm.diag >> gl) & 1u);
  const uint32_t my_m = pm.m[gl], my_ml = pm.ml[gl], my_mh = pm.mh[gl];
  double fl = 0.0;
  const uint32_t low = (1u << w0) - 1u;
  const int64_t step = (((int64_t)gridDim.x * blockDim.x) >> 5) * 32;
  int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
  uint32_t s_n = 0u;
  double x_n = 0.0;
  if (base + lane < dim) {
    s_n = states[base + lane];
    x_n = pr[base + lane];
  }
  for (; base < dim; base += step) {
    const int64_t r = base + lane;
    const bool valid = r < dim;
    const uint32_t s = s_n;
    const double x = x_n;
    s_n = 0u;  // rows past the end: never marked
    x_n = 0.0;
    if (base + step + lane < dim) {
      s_n = states[base + step + lane];
      x_n = pr[base + step + lane];
    }
    const uint32_t r0 = valid ? (uint32_t)t0s[s & low] : 0u;  // rank(s) = r0 + T1[s_hi]
    const uint32_t r1 = (uint32_t)r - r0;                    // = T1[s_hi]
    uint32_t L = 0u;
#pragma unroll
    for (int g = 0; g < MEAS_GR; ++g) {
      const bool lead = valid && g < pm.n && !((pm.diag >> g) & 1u) && (s & pm.m[g]) == pm.bi[g];
      const uint32_t bal = __ballot_sync(FULL, lead);
      L = gl == g ? bal : L;
    }
    if (!gl_on) L = 0u;
    if (par) L &= L - 1u;  // the pair's second lane starts at its second marked row
    const int mine = (__popc(L) + 1) >> 1;
    const int T = __reduce_max_sync(FULL, (unsigned)mine);
    for (int t = 0; t < T; t += FL_U) {
      int k[FL_U];
      bool has[FL_U];
#pragma unroll
      for (int u = 0; u < FL_U; ++u) {
        has[u] = L != 0u;
        k[u] = has[u] ? __ffs(L) - 1 : lane;
        L &= L - 1u;  // taken
        L &= L - 1u;  // the other lane's
      }
      double xk[FL_U], q[FL_U];
#pragma unroll
      for (int u = 0; u < FL_U; ++u) {
        const uint32_t sk = __shfl_sync(FULL, s, k[u]);
        const uint32_t r0k = __shfl_sync(FULL, r0, k[u]);
        const uint32_t r1k = __shfl_sync(FULL, r1, k[u]);
        xk[u] = __shfl_sync(FULL, x, k[u]);
        q[u] = 0.0;
        if (has[u]) {
          const uint32_t f = sk ^ my_m;
          const uint32_t c = (my_ml ? (uint32_t)t0s[f & low] : r0k) + (my_mh ? __ldg(&t1[f >> w0]) : r1k);
          q[u] = __ldg(&pr[c]);
        }
      }
#pragma unroll
      for (int u = 0; u < FL_U; ++u)
        if (has[u]) fl = fma(xk[u], q[u], fl);
    }
  }
  __shared__ double shf[8 * 32];
  shf[wid * 32 + lane] = fl;
  __syncthreads();
  if (threadIdx.x < MEAS_GR) {
    const int g = threadIdx.x;
    double a = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += shf[w * 32 + 2 * g] + shf[w * 32 + 2 * g + 1];
    partial[(size_t)(3 * g + 2) * nblk + blockIdx.x] = a;
  }
}

// Signed 128-bit (lo, hi) to the nearest double, approximately: |error| below
// 2^-52 of the value.
__device__ __forceinline__ double ed_i128_to_double(unsigned long long lo, unsigned long long hi) {
  const bool neg = (long long)hi < 0;
  if (neg) {  // magnitude
    lo = ~lo;
    hi = ~hi;
    ed_add128(lo, hi, 1ull, 0ull);
  }
  const double d = fma((double)hi, 0x1p64, (double)lo);
  return neg ? -d : d;
}

// out[g] from the block partials, summed in a fixed order (the integer ones
// exactly), F the flip sum, all integer sums times 2^-S:
//   S^z S^z: 0.25 (T - 2 A) (i != j), 0.25 T (i == j);
//   S.S:     0.25 (T - 2 A) + F (i != j), 0.75 T (i == j);
//   S+S-:    F (i != j), A (i == j: n_i);  S-S+: F (i != j), T - A (1 - n_i).
// One block per pair.
__global__ void k_expect_sym_finish(const double* __restrict__ partial, int nblk, const PairMasks pm, int op,
                                    double inv_scale, double* __restrict__ out) {
  const bool flips = op != ED_OP_SZSZ;
  const int g = blockIdx.x;
  if (g >= pm.n) return;
  __shared__ double shd[256];
  __shared__ unsigned long long sh[4][256];
  double a = 0.0;
  unsigned long long alo = 0ull, ahi = 0ull, tlo = 0ull, thi = 0ull;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    if (flips) a += partial[(size_t)(3 * g + 2) * nblk + b];
    ed_add128(alo, ahi, (unsigned long long)__double_as_longlong(partial[(size_t)(3 * g) * nblk + b]),
              (unsigned long long)__double_as_longlong(partial[(size_t)(3 * g + 1) * nblk + b]));
    ed_add128(tlo, thi, (unsigned long long)__double_as_longlong(partial[(size_t)(3 * MEAS_GR) * nblk + b]),
              (unsigned long long)__double_as_longlong(partial[(size_t)(3 * MEAS_GR + 1) * nblk + b]));
  }
  shd[threadIdx.x] = a;
  sh[0][threadIdx.x] = alo;
  sh[1][threadIdx.x] = ahi;
  sh[2][threadIdx.x] = tlo;
  sh[3][threadIdx.x] = thi;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      shd[threadIdx.x] += shd[threadIdx.x + st];
      unsigned long long l0 = sh[0][threadIdx.x], h0 = sh[1][threadIdx.x];
      ed_add128(l0, h0, sh[0][threadIdx.x + st], sh[1][threadIdx.x + st]);
      sh[0][threadIdx.x] = l0;
      sh[1][threadIdx.x] = h0;
      unsigned long long l1 = sh[2][threadIdx.x], h1 = sh[3][threadIdx.x];
      ed_add128(l1, h1, sh[2][threadIdx.x + st], sh[3][threadIdx.x + st]);
      sh[2][threadIdx.x] = l1;
      sh[3][threadIdx.x] = h1;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const bool diag = (pm.diag >> g) & 1u;
    const unsigned long long Alo = sh[0][0], Ahi = sh[1][0], Tlo = sh[2][0], Thi = sh[3][0];
    unsigned long long nlo = ~Alo, nhi = ~Ahi;
    ed_add128(nlo, nhi, 1ull, 0ull);  // -A
    double v;
    if (op == ED_OP_SZSZ || op == ED_OP_SISJ) {
      unsigned long long zlo = Tlo, zhi = Thi;  // Z = T - 2 A, |Z| <= T < 2^124 (A = 0 counts for i == j)
      if (!diag) {
        ed_add128(zlo, zhi, nlo, nhi);
        ed_add128(zlo, zhi, nlo, nhi);
      }
      v = 0.25 * (ed_i128_to_double(zlo, zhi) * inv_scale);
      if (op == ED_OP_SISJ) {
        if (diag) v += 0.5 * (ed_i128_to_double(Tlo, Thi) * inv_scale);  // (S+S- + S-S+) / 2
        else v += shd[0];
      }
    } else if (!diag) {
      v = shd[0];
    } else if (op == ED_OP_SPSM) {
      v = ed_i128_to_double(Alo, Ahi) * inv_scale;
    } else {
      unsigned long long dlo = Tlo, dhi = Thi;
      ed_add128(dlo, dhi, nlo, nhi);  // T - A
      v = ed_i128_to_double(dlo, dhi) * inv_scale;
    }
    out[g] = v;
  }
}

__global__ void k_real_parts(const double2* __restrict__ src, double* __restrict__ dst, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) dst[r] = src[r].x;
}

// ED_ENOMEM (nothing launched) when the compact copy does not fit, ED_ENOTSUP
// when psi is not finite: the general kernel then runs instead.
template <int OP>
static int expect_sym_r(const ed_basis* b, const double2* psi, const int32_t* pairs, int64_t np, double2* out) {
  ed_ctx* ctx = b->ctx;
  const int64_t dim = b->dim;
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((dim + 255) / 256, (int64_t)ctx->num_sms * 4));
  const size_t smem = sizeof(uint16_t) * ((size_t)1 << b->lin_w0);
  double* pr = nullptr;
  if (cudaMalloc(&pr, sizeof(double) * (size_t)dim) != cudaSuccess) {
    cudaGetLastError();  // clear the allocation failure
    return ED_ENOMEM;
  }
  int rc = ED_OK;
  {
    const int gs = (int)std::max<int64_t>(1, std::min<int64_t>((dim + 255) / 256, (int64_t)ctx->num_sms * 8));
    k_real_parts<<<gs, 256, 0, ctx->stream>>>(psi, pr, dim);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) rc = ed_cuda_fail(le, "k_real_parts launch", __FILE__, __LINE__);
    else ctx->kernels++;
  }
  // sum_r psi_r^2 = W < 2^e: every w_r and every integer sum stays below
  // 2^124 at the scale 2^(124 - e) (the rounding of W moves it by far less
  // than the spare bits)
  double W = 0.0;
  if (rc == ED_OK) rc = ed_multidot_r(ctx, nullptr, 0, pr, dim, nullptr, 0.0, nullptr, 0.0, nullptr, &W);
  if (rc == ED_OK && !std::isfinite(W)) rc = ED_ENOTSUP;
  int e = 0;
  if (rc == ED_OK && W > 0.0) std::frexp(W, &e);
  const int S = 124 - e;
  const double inv_scale = std::ldexp(1.0, -S);
  const size_t items = (size_t)3 * (MEAS_GR + 1);
  if (rc == ED_OK) rc = ed_ensure_reduce(ctx, items * nblk + MEAS_GR + 8);
  double* out_dev = ctx->d_red + items * nblk;
  const uint32_t low = (1u << b->lin_w0) - 1u;
  for (int64_t p0 = 0; p0 < np && rc == ED_OK; p0 += MEAS_GR) {
    PairMasks pm;
    memset(&pm, 0, sizeof(pm));
    pm.n = (int)std::min<int64_t>(MEAS_GR, np - p0);
    for (int g = 0; g < pm.n; ++g) {
      const int i = pairs[2 * (p0 + g)], j = pairs[2 * (p0 + g) + 1];
      const uint32_t m = (1u << i) | (1u << j);
      if (i == j) pm.diag |= 1u << g;
      pm.m[g] = m;
      pm.bi[g] = 1u << i;
      pm.ml[g] = m & low;
      pm.mh[g] = m >> b->lin_w0;
    }
    k_expect_zz_r<<<nblk, 256, 0, ctx->stream>>>(b->d_states, pr, dim, S, pm, ctx->d_red, nblk);
    cudaError_t le = cudaGetLastError();
    if (le == cudaSuccess) {
      ctx->kernels++;
      if (OP != ED_OP_SZSZ) {
        k_expect_flip_r<<<nblk, 256, smem, ctx->stream>>>(b->d_states, pr, dim, b->d_lin_t0, b->d_lin_t1,
                                                          b->lin_w0, pm, ctx->d_red, nblk);
        le = cudaGetLastError();
        if (le == cudaSuccess) ctx->kernels++;
      }
    }
    if (le == cudaSuccess) {
      k_expect_sym_finish<<<pm.n, 256, 0, ctx->stream>>>(ctx->d_red, nblk, pm, OP, inv_scale, out_dev);
      le = cudaGetLastError();
    }
    if (le == cudaSuccess) {
      ctx->kernels++;
      le = cudaMemcpyAsync(ctx->h_red, out_dev, sizeof(double) * pm.n, cudaMemcpyDeviceToHost, ctx->stream);
    }
    if (le == cudaSuccess) le = cudaStreamSynchronize(ctx->stream);
    if (le != cudaSuccess) {
      rc = ed_cuda_fail(le, "expectation pass", __FILE__, __LINE__);
      break;
    }
    for (int g = 0; g < pm.n; ++g) {
      out[p0 + g].x = ctx->h_red[g];
      out[p0 + g].y = 0.0;
    }
  }
  const cudaError_t fe = cudaFree(pr);
  if (fe != cudaSuccess && rc == ED_OK) rc = ed_cuda_fail(fe, "cudaFree", __FILE__, __LINE__);
  return rc;
}

int ed_launch_expect_pairs(const ed_basis* b, int op, const double2* psi, const int32_t* pairs, int64_t np,
                           double2* out) {
  bool real = false;
  ED_TRY(ed_is_real(b->ctx, psi, b->dim, &real));
  if (real) {
    int rc = ED_ENOTSUP;
    switch (op) {
      case ED_OP_SZSZ: rc = expect_sym_r<ED_OP_SZSZ>(b, psi, pairs, np, out); break;
      case ED_OP_SPSM: rc = expect_sym_r<ED_OP_SPSM>(b, psi, pairs, np, out); break;
      case ED_OP_SMSP: rc = expect_sym_r<ED_OP_SMSP>(b, psi, pairs, np, out); break;
      case ED_OP_SISJ: rc = expect_sym_r<ED_OP_SISJ>(b, psi, pairs, np, out); break;
      default: break;
    }
    if (rc != ED_ENOMEM && rc != ED_ENOTSUP) return rc;  // else the general kernel below
  }
  if (real) return expect_g<MEAS_GR, true>(b, op, psi, pairs, np, out);
  return expect_g<MEAS_G, false>(b, op, psi, pairs, np, out);
}

// ---------------------------------------------------------------------------
// DSF coefficients.  One launch handles up to MEAS_G sites for one target
// vector v_n.
//   Sqz: c_{i,n} = sum_r conj(v_n[r]) * 0.5 * (b_i(s_r) ? 1 : -1) * psi0[r]
//   Sqp: c_{i,n} = sum_{r: b_i(s_r) = 0} conj(v_n[rank1(s_r | 1<<i)]) * psi0[r]
// ---------------------------------------------------------------------------
template <int K1>
__global__ void __launch_bounds__(256) k_dsf(const uint32_t* __restrict__ states0, const double2* __restrict__ psi0,
                                             int64_t dim0, const RankTables rt1, int op, int i0, int ni,
                                             const double2* __restrict__ v, double* __restrict__ partial, int nblk) {
  extern __shared__ uint32_t stab[];
  if (op == 1) ed_load_tables(stab, rt1);
  double acc[2 * MEAS_G];
#pragma unroll
  for (int k = 0; k < 2 * MEAS_G; ++k) acc[k] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim0; r += stride) {
    const uint32_t s = states0[r];
    const double2 p = psi0[r];
    if (op == 0) {
      const double2 q = v[r];
      // conj(q) * p
      const double pr = fma(q.x, p.x, q.y * p.y), pi = fma(q.x, p.y, -q.y * p.x);
#pragma unroll
      for (int g = 0; g < MEAS_G; ++g) {
        if (g < ni) {
          const double sg = ((s >> (i0 + g)) & 1u) ? 0.5 : -0.5;
          acc[2 * g] = fma(sg, pr, acc[2 * g]);
          acc[2 * g + 1] = fma(sg, pi, acc[2 * g + 1]);
        }
      }
    } else {
#pragma unroll
      for (int g = 0; g < MEAS_G; ++g) {
        if (g < ni && !((s >> (i0 + g)) & 1u)) {
          const uint32_t c = ed_rank<K1>(s | (1u << (i0 + g)), stab, rt1);
          const double2 q = __ldg(&v[c]);
          acc[2 * g] += fma(q.x, p.x, q.y * p.y);
          acc[2 * g + 1] += fma(q.x, p.y, -q.y * p.x);
        }
      }
    }
  }
  __shared__ double sh[2 * MEAS_G * 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < 2 * MEAS_G; ++k) {
    double a = acc[k];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) sh[k * 32 + wid] = a;
  }
  __syncthreads();
  if (wid == 0) {
    for (int k = 0; k < 2 * MEAS_G; ++k) {
      double a = lane < nw ? sh[k * 32 + lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      if (lane == 0) partial[(size_t)k * nblk + blockIdx.x] = a;
    }
  }
}

template <int K1>
static int dsf_k(const ed_basis* b0, const ed_basis* b1, int op, const double2* psi0, const double2* vecs, int nev,
                 double2* c_host) {
  ed_ctx* ctx = b0->ctx;
  const int64_t dim0 = b0->dim, dim1 = b1->dim;
  const int N = b0->nspins;
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>((dim0 + 255) / 256, (int64_t)ctx->num_sms * 2));
  const int items = 2 * MEAS_G;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)items * nblk + items + 8));
  size_t smem = op == 1 ? (size_t)b1->rt.total * sizeof(uint32_t) : 0;
  ED_CUDA(cudaFuncSetAttribute(k_dsf<K1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(56 * 1024)));
  double* out_dev = ctx->d_red + (size_t)items * nblk;
  for (int n = 0; n < nev; ++n) {
    const double2* v = vecs + (size_t)n * dim1;
    for (int i0 = 0; i0 < N; i0 += MEAS_G) {
      int ni = std::min(MEAS_G, N - i0);
      k_dsf<K1><<<nblk, 256, smem, ctx->stream>>>(b0->d_states, psi0, dim0, b1->rt, op, i0, ni, v, ctx->d_red, nblk);
      ED_CHECK_LAUNCH(ctx);
      k_sum_partials<<<items, 256, 0, ctx->stream>>>(ctx->d_red, nblk, items, out_dev);
      ED_CHECK_LAUNCH(ctx);
      ED_CUDA(cudaMemcpyAsync(ctx->h_red, out_dev, sizeof(double) * items, cudaMemcpyDeviceToHost, ctx->stream));
      ED_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int g = 0; g < ni; ++g) {
        c_host[(size_t)(i0 + g) * nev + n].x = ctx->h_red[2 * g];
        c_host[(size_t)(i0 + g) * nev + n].y = ctx->h_red[2 * g + 1];
      }
    }
  }
  return ED_OK;
}

int ed_launch_dsf(const ed_basis* b0, const ed_basis* b1, int op, const double2* psi0, const double2* vecs, int nev,
                  double2* c_host) {
  switch (b1->rt.K) {
    case 1: return dsf_k<1>(b0, b1, op, psi0, vecs, nev, c_host);
    case 2: return dsf_k<2>(b0, b1, op, psi0, vecs, nev, c_host);
    case 3: return dsf_k<3>(b0, b1, op, psi0, vecs, nev, c_host);
    default: return dsf_k<4>(b0, b1, op, psi0, vecs, nev, c_host);
  }
}
