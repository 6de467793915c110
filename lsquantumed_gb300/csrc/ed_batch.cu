// Batched disorder sweep: B realisations of the same Hamiltonian that differ
// only in the random fields h_i (main_disorder.cpp:82-120 runs them one after
// another; build_disorder, hamiltonian.tmpl_func.hpp:97-125, rewrites only
// the diagonal).  All realisations share the off-diagonal pattern, so the
// batch is held as one [dim][B] array (realisation index fastest): a row's
// rank lookups serve all B columns and every gather reads B contiguous
// complex128 values.  B Krylov-Schur solves run in lockstep (same expansion
// and restart schedule), each with its own projected matrix and convergence;
// a realisation whose nev pairs have converged has its Ritz vectors saved and
// is frozen.
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

struct ed_batch {
  ed_ham* h = nullptr;
  int B = 0;
  int64_t dim = 0;
  double* d_diag = nullptr;        // [dim][B], build_disorder semantics per realisation
  longlong2* d_xq = nullptr;       // fixed-point copy of the SpMM input
  int* d_gmax = nullptr;
  // solver results
  int nev = 0, nrep = 0, its = 0;
  int64_t nhv = 0;
  std::vector<double> evals, errs;  // [B][nrep]
  std::vector<int> nconv;           // [B]
  double* d_vecs = nullptr;         // [nrep][dim][B] saved Ritz vectors (real parts)
  double* d_red = nullptr;
  size_t red_cap = 0;
  double* h_red = nullptr;
  int restart_arith = ED_RESTART_AUTO;  // ed_batch_set_restart_arithmetic
  int hv_variant = -1;  // batched H.v launch variant (-1: autotune at the next real-storage H.v)
  bool hv_forced = false;
  bool graphs = true;  // capture each expansion sweep after the first in a CUDA graph
  cudaStream_t stream = nullptr;  // the solve's own stream (ordered with the context's by events)
  int64_t graph_sweeps = 0;  // sweeps run from a captured graph in the last solve
};

// Per-realisation diagonal, exactly as build_disorder computes it:
// D1*0.25*E_nn + D2*0.25*E_nnn + 0.5*sum_i(+-h_i), separately rounded.
struct BatchDiagParams {
  int nb, N, B;
  uint32_t mask[ED_MAX_BONDS];
  uint8_t type[ED_MAX_BONDS];
  double D1, D2;
};

__global__ void k_batch_diag(const uint32_t* __restrict__ states, int64_t dim, const BatchDiagParams p,
                             const double* __restrict__ hi /* [B][N] */, double* __restrict__ diag) {
  const int64_t total = dim * p.B;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += stride) {
    const int64_t r = k / p.B;
    const int b = (int)(k - r * p.B);
    const uint32_t s = states[r];
    int n1 = 0, a1 = 0, n2 = 0, a2 = 0;
    for (int q = 0; q < p.nb; ++q) {
      const uint32_t t = s & p.mask[q];
      const int anti = (t != 0u && t != p.mask[q]) ? 1 : 0;
      if (p.type[q] == 0) { ++n1; a1 += anti; } else { ++n2; a2 += anti; }
    }
    double dis = 0.0;
    const double* h = hi + (size_t)b * p.N;
    for (int i = 0; i < p.N; ++i) dis = ((s >> i) & 1u) ? __dadd_rn(dis, h[i]) : __dsub_rn(dis, h[i]);
    const double x = __dmul_rn(__dmul_rn(p.D1, 0.25), (double)(n1 - 2 * a1));
    const double y = __dmul_rn(__dmul_rn(p.D2, 0.25), (double)(n2 - 2 * a2));
    diag[k] = __dadd_rn(__dadd_rn(x, y), __dmul_rn(0.5, dis));
  }
}

// Largest finite exponent over the batch array, for the fixed-point copy.
__global__ void k_batch_maxexp(const double2* __restrict__ x, int64_t n, int* __restrict__ gmax) {
  int m = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const double2 v = x[r];
    const int er = (int)(((unsigned long long)__double_as_longlong(v.x) >> 52) & 0x7FF);
    const int ei = (int)(((unsigned long long)__double_as_longlong(v.y) >> 52) & 0x7FF);
    m = max(m, max(er == 0x7FF ? 0 : er, ei == 0x7FF ? 0 : ei));
  }
  m = (int)__reduce_max_sync(0xffffffffu, (unsigned)m);
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(gmax, m);
}

__global__ void k_batch_quantize(const double2* __restrict__ x, int64_t n, const int* __restrict__ gmax_p, int sbits,
                                 longlong2* __restrict__ xq) {
  const int emax = *gmax_p;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const double2 v = x[r];
    const unsigned long long bits[2] = {(unsigned long long)__double_as_longlong(v.x),
                                        (unsigned long long)__double_as_longlong(v.y)};
    long long q[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int e = (int)((bits[k] >> 52) & 0x7FF);
      long long m = 0;
      if (e == 0x7FF) {
        m = (long long)0x8000000000000000ull;
      } else if (e != 0) {
        const unsigned long long mant = (bits[k] & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
        const int sh = e - emax + sbits - 53;
        unsigned long long a;
        if (sh >= 0) a = mant << sh;
        else if (sh > -63) a = (mant + (1ull << (-sh - 1))) >> (-sh);
        else a = 0;
        m = (long long)a;
        if (bits[k] >> 63) m = -m;
      }
      q[k] = m;
    }
    xq[r] = make_longlong2(q[0], q[1]);
  }
}

// The same two passes for the real-storage block of the batched solve.
__global__ void k_batch_maxexp_r(const double* __restrict__ x, int64_t n, int* __restrict__ gmax,
                                 const int* __restrict__ skip = nullptr) {
  if (skip && *skip) return;  // the fixed-point copy was made with x already
  int m = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
    const int e = (int)(((unsigned long long)__double_as_longlong(x[r]) >> 52) & 0x7FF);
    m = max(m, e == 0x7FF ? 0 : e);
  }
  m = (int)__reduce_max_sync(0xffffffffu, (unsigned)m);
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(gmax, m);
}

__device__ __forceinline__ long long batch_fx64_entry(double v, int emax, int sbits) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((bits >> 52) & 0x7FF);
  long long m = 0;
  if (e == 0x7FF) {
    m = (long long)0x8000000000000000ull;
  } else if (e != 0) {
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const int sh = e - emax + sbits - 53;
    unsigned long long a;
    if (sh >= 0) a = mant << sh;
    else if (sh > -63) a = (mant + (1ull << (-sh - 1))) >> (-sh);
    else a = 0;
    m = (long long)a;
    if (bits >> 63) m = -m;
  }
  return m;
}

__global__ void k_batch_quantize_r(const double* __restrict__ x, int64_t n, const int* __restrict__ gmax_p, int sbits,
                                   long long* __restrict__ xq, const int* __restrict__ skip = nullptr) {
  if (skip && *skip) return;
  const int emax = *gmax_p;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride)
    xq[r] = batch_fx64_entry(x[r], emax, sbits);
}

// Batched H.v over a [dim][B] block.  A CTA takes a tile of BH_ROWS rows:
// first one warp per row resolves the row's bonds (the antiparallel test and
// the two-table rank of the flipped state) and writes only the flipping
// ones to shared memory, compacted with warp ballots: first-type targets
// from the front of the row's list, second-type ones from the back.  Then
// each thread owns realisation columns b and gathers the B contiguous values
// of every listed target, four at a time so several loads are in flight,
// with no test or select per bond.  Exact int64 sums of the fixed-point
// input per coupling type, rounded once.
#define BH_NONE 0xFFFFFFFFu
// launch variants of the batched H.v: rows per tile x threads per block (the
// autotuner times each once per batch; all give bit-identical results)
static const int kBhRows[4] = {4, 8, 16, 32};
static const int kBhThreads[2] = {128, 256};
static const int kBhVariants = 8;  // v: rows kBhRows[v / 2], threads kBhThreads[v % 2]

struct BatchBonds {
  int nb;
  uint32_t mask[ED_MAX_BONDS];
  uint8_t type[ED_MAX_BONDS];
};

// RS: real storage (x, y double[dim][B], fixed-point copy int64[dim][B]);
// else complex128 blocks with (re, im) fixed-point pairs.
template <bool RS, int BH_ROWS>
__global__ void __launch_bounds__(256) k_batch_hv(const uint32_t* __restrict__ states, const double* __restrict__ diag,
                                                  const void* __restrict__ xv_, const void* __restrict__ xq_,
                                                  const int* __restrict__ gmax_p, int sbits, void* __restrict__ y_,
                                                  int64_t dim, int B, const uint16_t* __restrict__ t0,
                                                  const uint32_t* __restrict__ t1, int w0, const BatchBonds bb,
                                                  double c0, double c1, double* __restrict__ partial) {
  const double2* __restrict__ x = (const double2*)xv_;
  const longlong2* __restrict__ xq = (const longlong2*)xq_;
  const double* __restrict__ xr = (const double*)xv_;
  const long long* __restrict__ xqr = (const long long*)xq_;
  extern __shared__ uint32_t sm[];
  uint16_t* t0s = (uint16_t*)sm;                       // 2^w0 entries
  uint32_t* tgt = sm + ((1 << w0) + 1) / 2;            // [BH_ROWS][nb]
  // with partial (real storage only): per-realisation x^T y and ||y||^2 of
  // this CTA's rows, [2][B] doubles after the targets (8-byte aligned)
  double* dacc = (double*)(sm + ((((1 << w0) + 1) / 2 + BH_ROWS * bb.nb + 1) & ~1));
  for (int i = threadIdx.x; i < (1 << w0); i += blockDim.x) t0s[i] = t0[i];
  if (RS && partial)
    for (int i = threadIdx.x; i < 2 * B; i += blockDim.x) dacc[i] = 0.0;
  const int e_unit = *gmax_p - 1022 - sbits;
  const double s1 = __longlong_as_double((long long)(e_unit / 2 + 1023) << 52);
  const double s2 = __longlong_as_double((long long)(e_unit - e_unit / 2 + 1023) << 52);
  // real storage: the couplings carry the fixed-point scale 2^e_unit (a power
  // of two, so c * 2^e is exact where it stays normal and the results are
  // bit-identical): one conversion and one product per sum
  const bool fold = RS && e_unit > -900 && e_unit < 900;
  const double c0s = c0 * s1 * s2, c1s = c1 * s1 * s2;
  const long long kNaN = (long long)0x8000000000000000ull;
  const uint32_t low = (1u << w0) - 1u;
  const int nb = bb.nb;
  __shared__ int cnt[BH_ROWS][2];  // flipping bonds of each type in the tile's rows
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
  for (int64_t r0 = (int64_t)blockIdx.x * BH_ROWS; r0 < dim; r0 += (int64_t)gridDim.x * BH_ROWS) {
    __syncthreads();  // t0s ready / previous tile's targets consumed
    for (int rr = warp; rr < BH_ROWS; rr += nwarp) {
      uint32_t* tl = tgt + rr * nb;
      int n0 = 0, n1 = 0;
      const bool valid = r0 + rr < dim;
      const uint32_t s = valid ? states[r0 + rr] : 0u;
      for (int q0 = 0; q0 < nb; q0 += 32) {
        const int q = q0 + lane;
        bool on = false;
        uint32_t c = 0u;
        int ty = 0;
        if (valid && q < nb) {
          const uint32_t m = bb.mask[q], t = s & m;
          if (t != 0u && t != m) {
            const uint32_t f = s ^ m;
            c = (uint32_t)t0s[f & low] + __ldg(&t1[f >> w0]);
            on = true;
            ty = bb.type[q];
          }
        }
        const unsigned b0 = __ballot_sync(0xffffffffu, on && ty == 0);
        const unsigned b1 = __ballot_sync(0xffffffffu, on && ty != 0);
        const unsigned below = (1u << lane) - 1u;
        if (on && ty == 0) tl[n0 + __popc(b0 & below)] = c;
        if (on && ty != 0) tl[nb - 1 - (n1 + __popc(b1 & below))] = c;
        n0 += __popc(b0);
        n1 += __popc(b1);
      }
      if (lane == 0) {
        cnt[rr][0] = n0;
        cnt[rr][1] = n1;
      }
    }
    __syncthreads();
    const int nrows = (int)(dim - r0 < BH_ROWS ? dim - r0 : BH_ROWS);
    for (int rr = 0; rr < nrows; ++rr) {
      const uint32_t* tr = tgt + rr * nb;
      const int n0 = cnt[rr][0], n1 = cnt[rr][1];
      for (int b = threadIdx.x; b < B; b += blockDim.x) {
        long long a[4] = {0, 0, 0, 0};
        bool bad = false;
        // type 0: tr[0 .. n0), accumulators a[0], a[1]; type 1: tr[nb - n1 .. nb), a[2], a[3]
        for (int ty = 0; ty < 2; ++ty) {
          const int qb = ty ? nb - n1 : 0, qe = ty ? nb : n0;
          long long ar = 0, ai = 0;
          for (int q0 = qb; q0 < qe; q0 += 4) {
            if (RS) {
              long long v[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) v[u] = q0 + u < qe ? __ldg(&xqr[(size_t)tr[q0 + u] * B + b]) : 0ll;
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                bad |= v[u] == kNaN;
                ar += v[u];
              }
            } else {
              longlong2 v[4];
#pragma unroll
              for (int u = 0; u < 4; ++u)
                v[u] = q0 + u < qe ? __ldg(&xq[(size_t)tr[q0 + u] * B + b]) : make_longlong2(0, 0);
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                bad |= (v[u].x == kNaN) | (v[u].y == kNaN);
                ar += v[u].x;
                ai += v[u].y;
              }
            }
          }
          if (ty) { a[2] = ar; a[3] = ai; } else { a[0] = ar; a[1] = ai; }
        }
        const size_t k = (size_t)(r0 + rr) * B + b;
        const double d = diag[k];
        const double2 xv = RS ? make_double2(xr[k], 0.0) : x[k];
        double yr, yi = 0.0;
        if (fold) {
          yr = fma(d, xv.x, fma(c0s, (double)a[0], c1s * (double)a[2]));
        } else {
          const double s0r = (double)a[0] * s1 * s2, t1r = (double)a[2] * s1 * s2;
          yr = fma(d, xv.x, fma(c0, s0r, c1 * t1r));
          if (!RS) {
            const double s0i = (double)a[1] * s1 * s2, t1i = (double)a[3] * s1 * s2;
            yi = fma(d, xv.y, fma(c0, s0i, c1 * t1i));
          }
        }
        if (bad) { yr = __longlong_as_double(0x7FF8000000000000ll); yi = yr; }
        if (RS) {
          ((double*)y_)[k] = yr;
          if (partial) {  // column b belongs to this thread in every tile: no race
            dacc[b] = fma(xv.x, yr, dacc[b]);
            dacc[B + b] = fma(yr, yr, dacc[B + b]);
          }
        } else {
          ((double2*)y_)[k] = make_double2(yr, yi);
        }
      }
    }
  }
  if (RS && partial) {
    // partial[(item * B + b) * gridDim.x + blk], item 0 = x^T y, 1 = ||y||^2
    for (int b = threadIdx.x; b < B; b += blockDim.x) {
      partial[(size_t)b * gridDim.x + blockIdx.x] = dacc[b];
      partial[((size_t)B + b) * gridDim.x + blockIdx.x] = dacc[B + b];
    }
  }
}

// ---------------------------------------------------------------------------
// Column-wise (per realisation) linear algebra on [dim][B] arrays of the
// batched solve.  Its basis is exactly real (real start vectors, real H), so
// the block holds the real parts only (double[dim][B]).
// ---------------------------------------------------------------------------
struct BCols {
  const double* p[64];
};

// partial[(item * B + b) * nblk + blk]; items 0..nv-1 = V_i^T w, item nv = ||w||^2.
// A block takes a contiguous range of rows; its 256 threads are Bp column
// lanes (consecutive b: coalesced) times 256 / Bp row lanes, and the row
// lanes are summed in shared memory in a fixed order at the end.
#define BD_MAXV 16
#define BU_REG 16  // k_batch_update_norm keeps up to this many coefficients in registers
// With vj: first w <- w - a_b vj - bet_b vjm1 (coef = [a][B], [bet][B]),
// written back, in the same pass (the local Lanczos projection).
__global__ void __launch_bounds__(256) k_batch_dots(const BCols V, int nv, double* __restrict__ w, int64_t dim,
                                                    int B, int with_norm, double* __restrict__ partial, int nblk,
                                                    const double* __restrict__ vj, const double* __restrict__ vjm1,
                                                    const double* __restrict__ coef, const int* __restrict__ pred) {
  if (pred && *pred == 0) return;  // a pass the device decided to skip (uniform over the grid)
  __shared__ double sh[256 * (BD_MAXV + 1)];
  const int Bp = B >= 256 ? 256 : ((B + 31) / 32) * 32;
  const int S = 256 / Bp;  // row lanes
  const int lane_b = threadIdx.x % Bp, lane_r = threadIdx.x / Bp;
  const int64_t rows_per = (dim + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per, r1 = min(dim, r0 + rows_per);
  for (int b0 = 0; b0 < B; b0 += Bp) {
    const int b = b0 + lane_b;
    const bool act = lane_r < S && b < B;
    for (int i0 = 0; i0 < max(nv, 1); i0 += BD_MAXV) {
      const int ni = max(0, min(BD_MAXV, nv - i0));
      const bool norm = with_norm && i0 == 0;
      double acc[BD_MAXV + 1];
#pragma unroll
      for (int i = 0; i <= BD_MAXV; ++i) acc[i] = 0.0;
      if (act) {
        const bool local = vj && i0 == 0;
        const double ca = local ? coef[b] : 0.0, cb = local ? coef[B + b] : 0.0;
        for (int64_t r = r0 + lane_r; r < r1; r += S) {
          const size_t k = (size_t)r * B + b;
          double wv = w[k];
          if (local) {
            wv = fma(-ca, vj[k], wv);
            if (vjm1) wv = fma(-cb, vjm1[k], wv);
            w[k] = wv;
          }
#pragma unroll
          for (int i = 0; i < BD_MAXV; ++i)
            if (i < ni) acc[i] = fma(V.p[i0 + i][k], wv, acc[i]);
          if (norm) acc[BD_MAXV] = fma(wv, wv, acc[BD_MAXV]);
        }
      }
      __syncthreads();  // sh free
#pragma unroll
      for (int i = 0; i <= BD_MAXV; ++i) sh[i * 256 + threadIdx.x] = acc[i];
      __syncthreads();
      if (lane_r == 0 && b < B) {
        for (int i = 0; i <= BD_MAXV; ++i) {
          if (i < ni || (i == BD_MAXV && norm)) {
            double t = 0.0;
            for (int q = 0; q < S; ++q) t += sh[i * 256 + q * Bp + lane_b];
            const int item = i < BD_MAXV ? i0 + i : nv;
            partial[((size_t)item * B + b) * nblk + blockIdx.x] = t;
          }
        }
      }
    }
  }
}

// out[item] = sum_k partial[item * nblk + k]: one warp per item, lanes over k
// (coalesced), a fixed shuffle tree (the same order every run).
// Items below nsum are summed over the blocks, the others maximised.
__global__ void k_batch_reduce(const double* __restrict__ partial, int nblk, int64_t items, double* __restrict__ out,
                               int64_t nsum, const int* __restrict__ pred = nullptr) {
  if (pred && *pred == 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t it = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < items; it += nwarps) {
    const bool mx = it >= nsum;
    double a = 0.0;
    for (int k = lane; k < nblk; k += 32) {
      const double v = partial[(size_t)it * nblk + k];
      a = mx ? fmax(a, v) : a + v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v = __shfl_down_sync(0xffffffffu, a, o);
      a = mx ? fmax(a, v) : a + v;
    }
    if (lane == 0) out[it] = a;
  }
}

// w[:, b] <- w[:, b] - sum_i V_i[:, b] h[i][b]
__global__ void __launch_bounds__(256) k_batch_update(const BCols V, int nv, const double* __restrict__ h /* [nv][B] */,
                                                      double* __restrict__ w, int64_t dim, int B) {
  const int64_t n = dim * B;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const int b = (int)(k % B);
    double wv = w[k];
#pragma unroll 4
    for (int i = 0; i < nv; ++i) wv = fma(-V.p[i][k], h[(size_t)i * B + b], wv);
    w[k] = wv;
  }
}

// The same update with the new ||w[:, b]||^2 per realisation in the same pass:
// partial[b * nblk + blk] (blocks over row ranges, lanes as in k_batch_dots).
// partial[(B + b) * nblk + blk]: max_r |w[r, b]| over the block's rows.
template <bool REG>
__global__ void __launch_bounds__(256) k_batch_update_norm(const BCols V, int nv, const double* __restrict__ h,
                                                           double* __restrict__ w, int64_t dim, int B,
                                                           double* __restrict__ partial, int nblk,
                                                           const int* __restrict__ pred = nullptr) {
  if (pred && *pred == 0) return;
  __shared__ double sh[256], shm[256];
  const int Bp = B >= 256 ? 256 : ((B + 31) / 32) * 32;
  const int S = 256 / Bp;
  const int lane_b = threadIdx.x % Bp, lane_r = threadIdx.x / Bp;
  const int64_t rows_per = (dim + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per, r1 = min(dim, r0 + rows_per);
  for (int b0 = 0; b0 < B; b0 += Bp) {
    const int b = b0 + lane_b;
    double nrm = 0.0;
    unsigned int amax = 0u;  // high word of max |w[r, b]|
    if (lane_r < S && b < B) {
      if (REG) {
        // nv <= BU_REG: this realisation's coefficients in registers, two
        // rows per pass (two independent FMA chains)
        double hr[BU_REG];
#pragma unroll
        for (int i = 0; i < BU_REG; ++i) hr[i] = i < nv ? h[(size_t)i * B + b] : 0.0;
        for (int64_t r = r0 + lane_r; r < r1; r += 2 * S) {
          const int64_t rb = r + S;
          const bool has1 = rb < r1;
          const size_t k0 = (size_t)r * B + b, k1 = (size_t)rb * B + b;
          double w0 = w[k0], w1 = has1 ? w[k1] : 0.0;
#pragma unroll
          for (int i = 0; i < BU_REG; ++i) {
            if (i < nv) {
              w0 = fma(-V.p[i][k0], hr[i], w0);
              if (has1) w1 = fma(-V.p[i][k1], hr[i], w1);
            }
          }
          w[k0] = w0;
          nrm = fma(w0, w0, nrm);
          amax = ed_absmax_hi(amax, w0);
          if (has1) {
            w[k1] = w1;
            nrm = fma(w1, w1, nrm);
            amax = ed_absmax_hi(amax, w1);
          }
        }
      } else {
        for (int64_t r = r0 + lane_r; r < r1; r += S) {
          const size_t k = (size_t)r * B + b;
          double wv = w[k];
#pragma unroll 4
          for (int i = 0; i < nv; ++i) wv = fma(-V.p[i][k], h[(size_t)i * B + b], wv);
          w[k] = wv;
          nrm = fma(wv, wv, nrm);
          amax = ed_absmax_hi(amax, wv);
        }
      }
    }
    __syncthreads();
    sh[threadIdx.x] = nrm;
    shm[threadIdx.x] = ed_absmax_hi_value(amax);
    __syncthreads();
    if (lane_r == 0 && b < B) {
      double t = 0.0, mx = 0.0;
      for (int q = 0; q < S; ++q) {
        t += sh[q * Bp + lane_b];
        mx = fmax(mx, shm[q * Bp + lane_b]);
      }
      partial[(size_t)b * nblk + blockIdx.x] = t;
      partial[(size_t)(B + b) * nblk + blockIdx.x] = mx;
    }
  }
}

// dst[:, b] = src[:, b] * s[b]
__global__ void k_batch_scale(const double* __restrict__ src, double* __restrict__ dst, const double* __restrict__ s,
                              int64_t dim, int B) {
  const int64_t n = dim * B;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) dst[k] = src[k] * s[k % B];
}

// ---------------------------------------------------------------------------
// Device-side steps of the batched expansion: the per-realisation
// coefficients (the local Lanczos pair, the Gram-Schmidt dots, the norms, the
// refinement decision and the scale of the new vector) stay in device memory
// between the kernels, so an expansion sweep has no host round trip; alpha
// and beta ([b][m + 1], as on the host) go back once per restart.
// ---------------------------------------------------------------------------
struct BxState {
  double* alpha;  // [B][m1]
  double* beta;   // [B][m1]
  double* prevn;  // [B] norm before the pass (DGKS test)
  double* wmax;   // [B] high word of max |w[:, b]| after the last pass
  int* again;     // any realisation needs the refinement pass
  int* emax;      // largest exponent of the scaled block
  int* finite;    // emax determined for every realisation
  int* xq_valid;  // the fixed-point copy was made with the new vector
};

// res_hv[b] = v_j^T w: alpha_j and the local coefficients (a_b, beta_{j-1,b})
__global__ void k_bx_local(const double* __restrict__ res_hv, int A, int j, int m1, int three, BxState st,
                           double* __restrict__ coefL) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b == 0) *st.again = 0;
  if (b >= A) return;
  const double a = res_hv[b];
  st.alpha[(size_t)b * m1 + j] = a;
  coefL[b] = a;
  coefL[A + b] = three ? st.beta[(size_t)b * m1 + j - 1] : 0.0;
}

// After an update pass: res_upd = [||w||^2 per b, high word of max |w| per b],
// dots = [(j + 1)][A] the pass's coefficients.  The first pass's norm before
// the update is sqrt(||w||^2 + sum_i dots_i^2) (Pythagoras against the
// orthonormal basis).
__global__ void k_bx_post(const double* __restrict__ res_upd, const double* __restrict__ dots, int A, int j, int m1,
                          int first, BxState st, const int* __restrict__ pred) {
  if (pred && *pred == 0) return;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= A) return;
  st.alpha[(size_t)b * m1 + j] += dots[(size_t)j * A + b];
  const double n2 = res_upd[b];
  const double nw = sqrt(n2);
  st.beta[(size_t)b * m1 + j] = nw;
  double pv = st.prevn[b];
  if (first) {
    double s2 = n2;
    for (int i = 0; i <= j; ++i) {
      const double c = dots[(size_t)i * A + b];
      s2 += c * c;
    }
    pv = sqrt(s2);
  }
  if (nw < 0.7071067811865476 * pv) atomicOr(st.again, 1);
  st.prevn[b] = nw;
  st.wmax[b] = res_upd[A + b];
}

// ed_fx64_emax_scaled on the device: the biased exponent of fl(max |w| * s)
// where the high word of max |w| determines it, else -1.
__device__ __forceinline__ int bx_emax_scaled(double absmax_hi, double s) {
  const unsigned long long lb = (unsigned long long)__double_as_longlong(absmax_hi);
  const double u = __longlong_as_double((long long)(lb | 0xFFFFFFFFull));
  const double ml = absmax_hi * s, mu = u * s;
  if (!isfinite(ml) || !isfinite(mu) || !(s > 0.0)) return -1;
  const int el = (int)(((unsigned long long)__double_as_longlong(ml) >> 52) & 0x7FF);
  const int eu = (int)(((unsigned long long)__double_as_longlong(mu) >> 52) & 0x7FF);
  return el == eu ? el : -1;
}

// scale factors 1 / beta_j (0 keeps a zero column zero) and the largest
// exponent of the scaled block; one block
__global__ void __launch_bounds__(256) k_bx_scale(int A, int j, int m1, BxState st, double* __restrict__ sc) {
  __shared__ int sh_e[256], sh_f[256];
  int e = 0, f = 1;
  for (int b = threadIdx.x; b < A; b += blockDim.x) {
    const double nb = st.beta[(size_t)b * m1 + j];
    const double s = nb > 1e-300 ? 1.0 / nb : 0.0;
    sc[b] = s;
    if (s == 0.0) continue;
    const int eb = bx_emax_scaled(st.wmax[b], s);
    if (eb < 0) f = 0;
    else e = max(e, eb);
  }
  sh_e[threadIdx.x] = e;
  sh_f[threadIdx.x] = f;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sh_e[threadIdx.x] = max(sh_e[threadIdx.x], sh_e[threadIdx.x + o]);
      sh_f[threadIdx.x] = min(sh_f[threadIdx.x], sh_f[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *st.emax = sh_e[0];
    *st.finite = sh_f[0];
  }
}

// dst = src * s per realisation and, in the same pass, the fixed-point copy
// of dst for the next batched H.v (k_batch_quantize_r's values) with the
// largest exponent from the device (k_bx_scale): where that exponent is not
// determined, only the scaled vector is written and the next batched H.v
// quantizes it itself.
__global__ void k_bx_scale_quantize(const double* __restrict__ src, double* __restrict__ dst,
                                    const double* __restrict__ s, int64_t dim, int B, int sbits,
                                    long long* __restrict__ xq, int* __restrict__ gmax, BxState st) {
  const int finite = *st.finite, emax = *st.emax;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (finite) gmax[0] = emax;
    *st.xq_valid = finite;
  }
  const int64_t n = dim * B;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const double v = src[k] * s[k % B];
    dst[k] = v;
    if (finite) xq[k] = batch_fx64_entry(v, emax, sbits);
  }
}

// before a quantization the next H.v may need: reset the exponent maximum
__global__ void k_bx_prequant(int* __restrict__ gmax, const int* __restrict__ xq_valid) {
  if (!*xq_valid) gmax[0] = 0;
}

// out_c[:, b] = sum_i V_i[:, b] Y[b][i][c]   (Y real, m x l per realisation),
// outputs c0..c0+nc-1 (nc <= 8).  A block takes a tile of TB realisations
// (TB a power of two <= 32; thread = realisation b0 + t % TB, row offset
// t / TB) and stages their m x 8 coefficients in shared memory, so each
// coefficient is read from global memory once per block instead of once per
// entry; the basis loads stay coalesced (TB consecutive entries of a row).
// PAIR: products in float pairs on the FP32 units (ed_pair; storage and
// final sums FP64), Y given as float pairs; else FP64 FMA.
template <bool PAIR>
__global__ void __launch_bounds__(256) k_batch_restart(const BCols V, int m, const void* __restrict__ Yv, int l,
                                                       BCols out, int c0, int nc, int64_t dim, int B, int TB) {
  extern __shared__ double shYd[];  // [TB][m * 8 + 1] (the +1 staggers the banks)
  const int ld = m * 8 + 1;
  const int bl = threadIdx.x % TB, rsub = threadIdx.x / TB, rpb = blockDim.x / TB;
  const int b0 = blockIdx.x * TB;
  for (int t = threadIdx.x; t < TB * m * 8; t += blockDim.x) {
    const int tb = t / (m * 8), rem = t % (m * 8), i = rem / 8, q = rem % 8;
    const int b = b0 + tb;
    double y = 0.0;
    if (b < B && q < nc) {
      const size_t at = ((size_t)b * m + i) * l + c0 + q;
      y = PAIR ? __longlong_as_double(((const long long*)Yv)[at]) : ((const double*)Yv)[at];
    }
    shYd[tb * ld + rem] = y;
  }
  __syncthreads();
  const int b = b0 + bl;
  if (b >= B) return;
  const double* yb = shYd + bl * ld;
  for (int64_t row = (int64_t)blockIdx.y * rpb + rsub; row < dim; row += (int64_t)gridDim.y * rpb) {
    const int64_t k = row * B + b;
    if (PAIR) {
      float s[8], c[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) s[q] = c[q] = 0.0f;
      for (int i = 0; i < m; ++i) {
        const float2 v = ed_pair(V.p[i][k]);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (q < nc) {
            const unsigned long long u = (unsigned long long)__double_as_longlong(yb[i * 8 + q]);
            ed_pair_mac(v, make_float2(__uint_as_float((unsigned int)u), __uint_as_float((unsigned int)(u >> 32))),
                        s[q], c[q]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nc) ((double*)out.p[c0 + q])[k] = ed_pair_value(s[q], c[q]);
    } else {
      double ar[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) ar[q] = 0.0;
      for (int i = 0; i < m; ++i) {
        const double vx = V.p[i][k];
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (q < nc) ar[q] = fma(vx, yb[i * 8 + q], ar[q]);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nc) ((double*)out.p[c0 + q])[k] = ar[q];
    }
  }
}

// start vectors: every realisation starts from the real parts of the plain
// solver's seeded start vector
__global__ void k_batch_start(uint64_t seed, int64_t dim, int B, double* __restrict__ v) {
  const int64_t n = dim * B;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const uint64_t base = seed * 0xD1B54A32D192ED03ull;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const uint64_t i = (uint64_t)(k / B);
    const uint64_t h1 = ed_splitmix64(base + 2 * i);
    const double u1 = (double)(h1 >> 11) * (1.0 / 9007199254740992.0);
    v[k] = 2.0 * u1 - 1.0;
  }
}

// realisation b's column of a real [dim][B] array as a complex128 vector
__global__ void k_batch_extract(const double* __restrict__ src, int64_t dim, int B, int b, double2* __restrict__ dst) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride)
    dst[r] = make_double2(src[(size_t)r * B + b], 0.0);
}

// dst[r][t] = src[r][keep[t]]: realisation columns keep[0..A2) of a [dim][A]
// array packed into a [dim][A2] array (the active set after convergence).
template <typename T>
__global__ void k_batch_pack(const T* __restrict__ src, T* __restrict__ dst, int64_t dim, int A, int A2,
                             const int* __restrict__ keep) {
  const int64_t n = dim * A2;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const int64_t r = k / A2;
    dst[k] = src[(size_t)r * A + keep[k % A2]];
  }
}

// dst[r][orig[t]] = src[r][slot[t]]: converged slots of a [dim][A] array into
// their realisations' columns of a [dim][B] array.
__global__ void k_batch_save(const double* __restrict__ src, double* __restrict__ dst, int64_t dim, int A, int B,
                             const int* __restrict__ slot, const int* __restrict__ orig, int ns) {
  const int64_t n = dim * ns;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const int64_t r = k / ns;
    const int t = (int)(k % ns);
    dst[(size_t)r * B + orig[t]] = src[(size_t)r * A + slot[t]];
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int grid_n(ed_ctx* ctx, int64_t n, int per_sm = 8) {
  int64_t g = (n + 255) / 256;
  int64_t cap = (int64_t)ctx->num_sms * per_sm;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

static int batch_reduce_buf(ed_batch* bt, size_t doubles) {
  if (doubles <= bt->red_cap) return ED_OK;
  if (bt->d_red) cudaFree(bt->d_red);
  if (bt->h_red) cudaFreeHost(bt->h_red);
  bt->d_red = nullptr;
  bt->h_red = nullptr;
  ED_CUDA(cudaMalloc(&bt->d_red, doubles * sizeof(double)));
  ED_CUDA(cudaMallocHost(&bt->h_red, doubles * sizeof(double)));
  bt->red_cap = doubles;
  return ED_OK;
}

// dots of nv real columns against w, per realisation; out (host) [item][B]:
// item i < nv = V_i^T w, item nv = ||w||^2.
static int batch_dots(ed_batch* bt, int B, const std::vector<const double*>& V, double* w, bool norm,
                      std::vector<double>& out, const double* vj = nullptr, const double* vjm1 = nullptr,
                      const double* coef = nullptr) {
  ed_ctx* ctx = bt->h->ctx;
  const int nv = (int)V.size();
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(bt->dim / 64 + 1, (int64_t)ctx->num_sms * 4));
  const int64_t items = (int64_t)(nv + 1) * B;
  ED_TRY(batch_reduce_buf(bt, (size_t)items * nblk + (size_t)items));
  BCols vc;
  memset(&vc, 0, sizeof(vc));
  for (int i = 0; i < nv && i < 64; ++i) vc.p[i] = V[i];
  k_batch_dots<<<nblk, 256, 0, ctx->stream>>>(vc, nv, w, bt->dim, B, norm ? 1 : 0, bt->d_red, nblk, vj, vjm1, coef,
                                              nullptr);
  ED_CHECK_LAUNCH(ctx);
  double* res = bt->d_red + (size_t)items * nblk;
  k_batch_reduce<<<grid_n(ctx, items * 32, 8), 256, 0, ctx->stream>>>(bt->d_red, nblk, items, res, items);
  ED_CHECK_LAUNCH(ctx);
  ED_CUDA(cudaMemcpyAsync(bt->h_red, res, sizeof(double) * (size_t)items, cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  out.assign(bt->h_red, bt->h_red + items);
  return ED_OK;
}

// The dots V_i^T w of a pass, reduced straight into out_dev ([nv][B], the
// update's coefficient layout), without a host round trip; pred (device):
// skip the pass when it reads 0.
static int batch_dots_dev(ed_batch* bt, int B, const std::vector<const double*>& V, double* w, double* out_dev,
                          const double* vj, const double* vjm1, const double* coef, const int* pred) {
  ed_ctx* ctx = bt->h->ctx;
  const int nv = (int)V.size();
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(bt->dim / 64 + 1, (int64_t)ctx->num_sms * 4));
  const int64_t items = (int64_t)nv * B;
  ED_TRY(batch_reduce_buf(bt, (size_t)(items + B) * nblk + (size_t)items));
  BCols vc;
  memset(&vc, 0, sizeof(vc));
  for (int i = 0; i < nv && i < 64; ++i) vc.p[i] = V[i];
  k_batch_dots<<<nblk, 256, 0, ctx->stream>>>(vc, nv, w, bt->dim, B, 0, bt->d_red, nblk, vj, vjm1, coef, pred);
  ED_CHECK_LAUNCH(ctx);
  k_batch_reduce<<<grid_n(ctx, items * 32, 8), 256, 0, ctx->stream>>>(bt->d_red, nblk, items, out_dev, items, pred);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

// Scale of the fixed-point H.v input (depends on the bond counts only).
static int batch_sbits(const ed_batch* bt) {
  const ed_ham* h = bt->h;
  int cnt[2] = {0, 0};
  for (int q = 0; q < h->bs.nb; ++q) cnt[h->bs.type[q] & 1]++;
  int head = 0;
  while ((1 << head) < std::max(cnt[0], cnt[1]) + 1) ++head;
  return 62 - head;
}

// y = H_b x for the B (active) realisation columns of x, whose diagonals are
// the columns of diag ([dim][B]).  rs: x, y are real storage double[dim][B]
// (the solve), else complex128 blocks (ed_batch_apply).
// dev (real storage only): the expansion's device state; the fixed-point copy
// is then made here only where the previous step could not (xq_valid), and
// with res_dev the fused x^T y / ||y||^2 stay on the device (*res_dev, in the
// reduce buffer, valid until its next use) instead of coming back to *dot.
static int batch_hv(ed_batch* bt, int B, const double* diag, const void* x, void* y, bool rs,
                    std::vector<double>* dot = nullptr, const BxState* dev = nullptr,
                    const double** res_dev = nullptr) {
  ed_ham* h = bt->h;
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  const int64_t n = bt->dim * B;
  const int sbits = batch_sbits(bt);
  if (rs && dev) {
    k_bx_prequant<<<1, 1, 0, ctx->stream>>>(bt->d_gmax, dev->xq_valid);
    ED_CHECK_LAUNCH(ctx);
    k_batch_maxexp_r<<<grid_n(ctx, n), 256, 0, ctx->stream>>>((const double*)x, n, bt->d_gmax, dev->xq_valid);
    ED_CHECK_LAUNCH(ctx);
    k_batch_quantize_r<<<grid_n(ctx, n), 256, 0, ctx->stream>>>((const double*)x, n, bt->d_gmax, sbits,
                                                                 (long long*)bt->d_xq, dev->xq_valid);
    ED_CHECK_LAUNCH(ctx);
  } else if (rs) {
    ED_CUDA(cudaMemsetAsync(bt->d_gmax, 0, sizeof(int), ctx->stream));
    k_batch_maxexp_r<<<grid_n(ctx, n), 256, 0, ctx->stream>>>((const double*)x, n, bt->d_gmax);
    ED_CHECK_LAUNCH(ctx);
    k_batch_quantize_r<<<grid_n(ctx, n), 256, 0, ctx->stream>>>((const double*)x, n, bt->d_gmax, sbits,
                                                                 (long long*)bt->d_xq);
    ED_CHECK_LAUNCH(ctx);
  } else {
    ED_CUDA(cudaMemsetAsync(bt->d_gmax, 0, sizeof(int), ctx->stream));
    k_batch_maxexp<<<grid_n(ctx, n), 256, 0, ctx->stream>>>((const double2*)x, n, bt->d_gmax);
    ED_CHECK_LAUNCH(ctx);
    k_batch_quantize<<<grid_n(ctx, n), 256, 0, ctx->stream>>>((const double2*)x, n, bt->d_gmax, sbits, bt->d_xq);
    ED_CHECK_LAUNCH(ctx);
  }
  BatchBonds bb;
  memset(&bb, 0, sizeof(bb));
  for (int q = 0; q < h->bs.nb; ++q) {
    if (__builtin_popcount(h->bs.mask[q]) != 2) continue;  // i == j never couples
    bb.mask[bb.nb] = h->bs.mask[q];
    bb.type[bb.nb] = (uint8_t)(h->bs.type[q] & 1);
    ++bb.nb;
  }
  // one launch of variant v; partial (real storage only): fused x^T y, ||y||^2
  auto launch = [&](int v, double* partial, int* grid_out) -> int {
    const int rows = kBhRows[v / 2];
    size_t smem = sizeof(uint32_t) * ((((size_t)1 << b->lin_w0) + 1) / 2 + (size_t)rows * std::max(bb.nb, 1));
    if (partial) smem = ((smem + 7) & ~(size_t)7) + sizeof(double) * 2 * (size_t)B + 8;
    if (smem > 96 * 1024) return ED_ENOTSUP;
    const int threads = std::min(kBhThreads[v % 2], ((B + 31) / 32) * 32);
    const void* fn = nullptr;
#define ED_BH_FN(R)                                                                  \
  case R:                                                                            \
    fn = rs ? (const void*)k_batch_hv<true, R> : (const void*)k_batch_hv<false, R>; \
    break;
    switch (rows) { ED_BH_FN(4) ED_BH_FN(8) ED_BH_FN(16) ED_BH_FN(32) }
#undef ED_BH_FN
    static std::atomic<bool> attr_set[2][4] = {};  // several host threads may launch (ed_batch_solve_many)
    std::atomic<bool>& done = attr_set[rs ? 1 : 0][v / 2];
    if (!done.load()) {
      ED_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
      done.store(true);
    }
    int per_sm = 0;
    ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    if (per_sm < 1) per_sm = 1;
    const int64_t tiles = (bt->dim + rows - 1) / rows;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)ctx->num_sms * per_sm));
    if (grid_out) *grid_out = grid;
    if (partial) ED_TRY(batch_reduce_buf(bt, (size_t)2 * B * grid + (size_t)2 * B));
    double* part = partial ? bt->d_red : nullptr;
#define ED_BH_LAUNCH(R)                                                                                             \
  case R:                                                                                                           \
    if (rs)                                                                                                         \
      k_batch_hv<true, R><<<grid, threads, smem, ctx->stream>>>(b->d_states, diag, x, bt->d_xq, bt->d_gmax, sbits, \
                                                                y, bt->dim, B, b->d_lin_t0, b->d_lin_t1,            \
                                                                b->lin_w0, bb, h->bs.chalf[0], h->bs.chalf[1],      \
                                                                part);                                              \
    else                                                                                                            \
      k_batch_hv<false, R><<<grid, threads, smem, ctx->stream>>>(b->d_states, diag, x, bt->d_xq, bt->d_gmax,       \
                                                                 sbits, y, bt->dim, B, b->d_lin_t0, b->d_lin_t1,   \
                                                                 b->lin_w0, bb, h->bs.chalf[0], h->bs.chalf[1],    \
                                                                 nullptr);                                          \
    break;
    switch (rows) { ED_BH_LAUNCH(4) ED_BH_LAUNCH(8) ED_BH_LAUNCH(16) ED_BH_LAUNCH(32) }
#undef ED_BH_LAUNCH
    ED_CHECK_LAUNCH(ctx);
    return ED_OK;
  };
  if (bt->hv_variant < 0 && rs) {
    // a batch of this width on this operator was tuned before: reuse
    for (const auto& t : h->batch_tile)
      if (t.first == B) bt->hv_variant = t.second;
  }
  if (bt->hv_variant < 0 && rs) {
    // time every variant on this input (plain H.v; the result is the same for
    // all of them), best of three launches each, and keep the fastest for
    // the batch's life and for later batches of this width on this operator
    cudaEvent_t e0, e1;
    ED_CUDA(cudaEventCreate(&e0));
    ED_CUDA(cudaEventCreate(&e1));
    float best = 0.0f;
    bool have = false;
    int vbest = 3;  // 8 rows x 256 threads
    for (int v = 0; v < kBhVariants; ++v) {
      int r = launch(v, nullptr, nullptr);  // warm-up (and the T0 fill of a new shape)
      if (r == ED_ENOTSUP) continue;
      ED_TRY(r);
      float ms = 0.0f;
      for (int rep = 0; rep < 3; ++rep) {
        ED_CUDA(cudaEventRecord(e0, ctx->stream));
        ED_TRY(launch(v, nullptr, nullptr));
        ED_CUDA(cudaEventRecord(e1, ctx->stream));
        ED_CUDA(cudaEventSynchronize(e1));
        float t = 0.0f;
        ED_CUDA(cudaEventElapsedTime(&t, e0, e1));
        if (rep == 0 || t < ms) ms = t;
      }
      if (!have || ms < best) {
        have = true;
        best = ms;
        vbest = v;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    bt->hv_variant = vbest;
    h->batch_tile.emplace_back(B, vbest);
  }
  const int v = bt->hv_variant < 0 ? 3 : bt->hv_variant;
  int grid = 0;
  {
    const int r = launch(v, (dot || res_dev) ? bt->d_red : nullptr, &grid);
    if (r == ED_ENOTSUP) return ed_fail(ED_ENOTSUP, "batch too wide for the batched H.v");
    ED_TRY(r);
  }
  if (dot || res_dev) {
    const int64_t items = 2 * (int64_t)B;
    double* res = bt->d_red + (size_t)items * grid;
    k_batch_reduce<<<grid_n(ctx, items * 32, 8), 256, 0, ctx->stream>>>(bt->d_red, grid, items, res, items);
    ED_CHECK_LAUNCH(ctx);
    if (res_dev) {
      *res_dev = res;
      return ED_OK;
    }
    ED_CUDA(cudaMemcpyAsync(bt->h_red, res, sizeof(double) * (size_t)items, cudaMemcpyDeviceToHost, ctx->stream));
    ED_CUDA(cudaStreamSynchronize(ctx->stream));
    if (dot) dot->assign(bt->h_red, bt->h_red + items);
  }
  return ED_OK;
}

extern "C" {

int ed_batch_create(ed_ham* h, int B, const double* hi_host, ed_batch** out) {
  if (!h || !hi_host || !out) return ed_fail(ED_EINVAL, "null argument");
  if (B < 1) return ed_fail(ED_EINVAL, "batch size must be >= 1");
  if (h->per_bond) return ed_fail(ED_ENOTSUP, "batched sweeps need uniform J1/J2 couplings");
  if (!h->offdiag_built) return ed_fail(ED_ESTATE, "build_off_diag before creating a batch");
  ed_ctx* ctx = h->ctx;
  const int N = h->basis->nspins;
  ed_batch* bt = new ed_batch();
  bt->h = h;
  bt->B = B;
  bt->dim = h->basis->dim;
  const size_t n = (size_t)bt->dim * B;
  double* dhi = nullptr;
  if (cudaMalloc(&bt->d_diag, sizeof(double) * n) != cudaSuccess || cudaMalloc(&bt->d_xq, sizeof(longlong2) * n) != cudaSuccess ||
      cudaMalloc(&bt->d_gmax, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&dhi, sizeof(double) * (size_t)B * N) != cudaSuccess) {
    cudaGetLastError();
    if (dhi) cudaFree(dhi);
    ed_batch_destroy(bt);
    return ed_fail(ED_ENOMEM, "batch does not fit in device memory");
  }
  cudaMemcpyAsync(dhi, hi_host, sizeof(double) * (size_t)B * N, cudaMemcpyHostToDevice, ctx->stream);
  BatchDiagParams p;
  memset(&p, 0, sizeof(p));
  p.nb = (int)h->bi.size();
  p.N = N;
  p.B = B;
  p.D1 = h->D1;
  p.D2 = h->D2;
  for (int q = 0; q < p.nb; ++q) {
    p.mask[q] = (1u << h->bi[q]) | (1u << h->bj[q]);
    p.type[q] = (uint8_t)h->btype[q];
  }
  k_batch_diag<<<grid_n(ctx, (int64_t)n), 256, 0, ctx->stream>>>(h->basis->d_states, bt->dim, p, dhi, bt->d_diag);
  cudaError_t e = cudaGetLastError();
  cudaStreamSynchronize(ctx->stream);
  cudaFree(dhi);
  if (e != cudaSuccess) {
    ed_batch_destroy(bt);
    return ed_cuda_fail(e, "k_batch_diag", __FILE__, __LINE__);
  }
  ctx->kernels++;
  *out = bt;
  return ED_OK;
}

int ed_batch_destroy(ed_batch* bt) {
  if (!bt) return ED_OK;
  if (bt->d_diag) cudaFree(bt->d_diag);
  if (bt->d_xq) cudaFree(bt->d_xq);
  if (bt->d_gmax) cudaFree(bt->d_gmax);
  if (bt->d_vecs) cudaFree(bt->d_vecs);
  if (bt->d_red) cudaFree(bt->d_red);
  if (bt->h_red) cudaFreeHost(bt->h_red);
  if (bt->stream) cudaStreamDestroy(bt->stream);
  delete bt;
  return ED_OK;
}

int ed_batch_apply(ed_batch* bt, const ed_cplx* x_dev, ed_cplx* y_dev) {
  if (!bt || !x_dev || !y_dev) return ed_fail(ED_EINVAL, "null argument");
  if ((const void*)x_dev == (const void*)y_dev) return ed_fail(ED_EINVAL, "x and y must not alias");
  return batch_hv(bt, bt->B, bt->d_diag, x_dev, y_dev, false);
}

int ed_batch_diag_host(ed_batch* bt, double* out_host) {
  if (!bt || !out_host) return ed_fail(ED_EINVAL, "null argument");
  ED_CUDA(cudaMemcpyAsync(out_host, bt->d_diag, sizeof(double) * (size_t)bt->dim * bt->B, cudaMemcpyDeviceToHost,
                          bt->h->ctx->stream));
  ED_CUDA(cudaStreamSynchronize(bt->h->ctx->stream));
  return ED_OK;
}

// Lockstep Krylov-Schur over the batch (same method as ed_eps_solve: local
// Lanczos projection + one CGS pass with the DGKS refinement test, thick
// restart keeping l = max(nev + 2, ncv / 2) vectors), with exact real
// arithmetic (real start vectors, real H).  At every restart the
// realisations whose nev pairs converged save their Ritz vectors and leave
// the active block, which is packed to the remaining A columns, so the work
// follows the sum of the realisations' iterations, not B times the slowest.
static int batch_solve_impl(ed_batch* bt, int nev, int ncv, double tol, int max_it, uint64_t seed,
                            double* evals_host, double* errs_host, int* nconv_host);

// The solve runs on the batch's own non-blocking stream, ordered after the
// context stream's earlier work and before its later work by events: batches
// of different environments then overlap on the device even when the
// environments use the legacy default stream, and a sweep can be captured in
// a CUDA graph (the legacy stream cannot be captured).
int ed_batch_solve(ed_batch* bt, int nev, int ncv, double tol, int max_it, uint64_t seed, double* evals_host,
                   double* errs_host, int* nconv_host) {
  if (!bt || !evals_host || !errs_host || !nconv_host) return ed_fail(ED_EINVAL, "null argument");
  ed_ctx* ctx = bt->h->ctx;
  if (!bt->stream) ED_CUDA(cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking));
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  ED_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
  if (cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming) != cudaSuccess) {
    cudaEventDestroy(ev_in);
    return ed_cuda_fail(cudaGetLastError(), "cudaEventCreate", __FILE__, __LINE__);
  }
  cudaStream_t outer = ctx->stream;
  int rc = ED_OK;
  if (cudaEventRecord(ev_in, outer) != cudaSuccess || cudaStreamWaitEvent(bt->stream, ev_in, 0) != cudaSuccess) {
    rc = ed_cuda_fail(cudaGetLastError(), "stream ordering", __FILE__, __LINE__);
  } else {
    ctx->stream = bt->stream;
    rc = batch_solve_impl(bt, nev, ncv, tol, max_it, seed, evals_host, errs_host, nconv_host);
    ctx->stream = outer;
    if (cudaEventRecord(ev_out, bt->stream) != cudaSuccess || cudaStreamWaitEvent(outer, ev_out, 0) != cudaSuccess)
      if (rc == ED_OK) rc = ed_cuda_fail(cudaGetLastError(), "stream ordering", __FILE__, __LINE__);
  }
  cudaEventDestroy(ev_in);
  cudaEventDestroy(ev_out);
  return rc;
}

static int batch_solve_impl(ed_batch* bt, int nev, int ncv, double tol, int max_it, uint64_t seed,
                            double* evals_host, double* errs_host, int* nconv_host) {
  ed_ctx* ctx = bt->h->ctx;
  const int64_t dim = bt->dim;
  const int B = bt->B;
  if (nev < 1) return ed_fail(ED_EINVAL, "nev must be >= 1");
  int m = ncv > 0 ? ncv : std::max(2 * nev, nev + 15);
  if (m > dim) m = (int)dim;
  if (nev > m) nev = m;
  if (m > 62) return ed_fail(ED_ENOTSUP, "batched ncv above 62 is not supported");
  if (m < nev + 2 && m < dim) m = std::min<int>((int)dim, nev + 2);
  if (tol <= 0) tol = 1e-8;
  if (max_it <= 0) max_it = (int)std::max<int64_t>(100, 2 * dim / std::max(m, 1));
  const int l_keep = std::min(m - 1, std::max(nev + 2, m / 2));
  const size_t colB = (size_t)dim * B;
  const int pool_cols = 2 * m + 1;
  double* pool = nullptr;
  double* w = nullptr;
  double* dg[2] = {nullptr, nullptr};
  double* d_coef = nullptr;  // [64][B] double2 coefficients / scale factors
  int* d_idx = nullptr;      // [2][B] slot / realisation index lists
  double* dY = nullptr;
  if (cudaMalloc(&pool, sizeof(double) * colB * pool_cols) != cudaSuccess ||
      cudaMalloc(&w, sizeof(double) * colB) != cudaSuccess || cudaMalloc(&dg[0], sizeof(double) * colB) != cudaSuccess ||
      cudaMalloc(&dg[1], sizeof(double) * colB) != cudaSuccess ||
      cudaMalloc(&d_coef, sizeof(double2) * 64 * (size_t)B) != cudaSuccess ||
      cudaMalloc(&d_idx, sizeof(int) * 2 * (size_t)B) != cudaSuccess ||
      cudaMalloc(&dY, sizeof(double) * (size_t)B * m * l_keep) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(pool); cudaFree(w); cudaFree(dg[0]); cudaFree(dg[1]); cudaFree(d_coef); cudaFree(d_idx); cudaFree(dY);
    return ed_fail(ED_ENOMEM, "batched Krylov basis does not fit in device memory");
  }
  if (bt->d_vecs) cudaFree(bt->d_vecs);
  bt->d_vecs = nullptr;
  if (cudaMalloc(&bt->d_vecs, sizeof(double) * colB * nev) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(pool); cudaFree(w); cudaFree(dg[0]); cudaFree(dg[1]); cudaFree(d_coef); cudaFree(d_idx); cudaFree(dY);
    return ed_fail(ED_ENOMEM, "batched eigenvectors do not fit in device memory");
  }
  // device state of the expansion sweeps
  BxState st;
  double* st_buf = nullptr;
  int* st_int = nullptr;
  const size_t m1 = (size_t)m + 1;
  if (cudaMalloc(&st_buf, sizeof(double) * (2 * m1 + 2) * (size_t)B) != cudaSuccess ||
      cudaMalloc(&st_int, sizeof(int) * 8) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(st_buf);
    cudaFree(pool); cudaFree(w); cudaFree(dg[0]); cudaFree(dg[1]); cudaFree(d_coef); cudaFree(d_idx); cudaFree(dY);
    return ed_fail(ED_ENOMEM, "batched solver state does not fit in device memory");
  }
  st.alpha = st_buf;
  st.beta = st_buf + m1 * B;
  st.prevn = st_buf + 2 * m1 * B;
  st.wmax = st_buf + (2 * m1 + 1) * B;
  st.again = st_int;
  st.emax = st_int + 1;
  st.finite = st_int + 2;
  st.xq_valid = st_int + 3;
  ED_CUDA(cudaMemsetAsync(st_int, 0, sizeof(int) * 8, ctx->stream));
  std::vector<double> st_host(2 * m1 * (size_t)B);
  std::vector<double*> col(m + 1), freel;
  for (int i = 0; i < pool_cols; ++i) {
    double* p = pool + (size_t)i * colB;
    if (i <= m) col[i] = p; else freel.push_back(p);
  }
  int cur = 0;  // dg[cur] holds the active realisations' diagonals
  int rc = ED_OK;
  bool capturing = false;  // the stream is capturing an expansion sweep
  bt->graph_sweeps = 0;
  std::vector<double> out;
  std::vector<double> alpha((size_t)B * (m + 1)), beta((size_t)B * (m + 1)), arrow((size_t)B * (m + 1));
  std::vector<int> act(B), nconv(B, 0);
  for (int b = 0; b < B; ++b) act[b] = b;
  bt->evals.assign((size_t)B * nev, 0.0);
  bt->errs.assign((size_t)B * nev, 0.0);
  std::vector<double> Yall;
  int k = 0, its = 0, A = B;
  bt->nhv = 0;
  ED_CUDA(cudaMemcpyAsync(dg[0], bt->d_diag, sizeof(double) * colB, cudaMemcpyDeviceToDevice, ctx->stream));
  // start vectors, normalised per realisation
  k_batch_start<<<grid_n(ctx, (int64_t)colB), 256, 0, ctx->stream>>>(seed, dim, A, col[0]);
  ctx->kernels++;
  {
    std::vector<const double*> none;
    if ((rc = batch_dots(bt, A, none, col[0], true, out)) != ED_OK) goto cleanup;
    std::vector<double> sc(A);
    for (int b = 0; b < A; ++b) sc[b] = 1.0 / std::sqrt(out[b]);
    cudaMemcpyAsync(d_coef, sc.data(), sizeof(double) * A, cudaMemcpyHostToDevice, ctx->stream);
    k_batch_scale<<<grid_n(ctx, (int64_t)dim * A), 256, 0, ctx->stream>>>(col[0], col[0], d_coef, dim, A);
    ctx->kernels++;
  }
  while (A > 0 && its < max_it) {
    ++its;
    const int64_t colA = dim * (int64_t)A;
    // the expansion sweep runs without a host round trip: the coefficients
    // live in the device state (st), alpha and beta come back after it.
    // With graphs on, the sweeps after the first (which tunes the H.v and
    // sizes the buffers) are captured in a CUDA graph and replayed once.
    bool capture = bt->graphs && its > 1;
    if (capture) {
      const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(dim / 64 + 1, (int64_t)ctx->num_sms * 4));
      const size_t nd = (size_t)m * A;
      const size_t need = std::max({(nd + A) * nblk + nd, (size_t)2 * A * nblk + 2 * (size_t)A,
                                    (size_t)2 * A * ((size_t)ctx->num_sms * 64) + 2 * (size_t)A});
      if ((rc = batch_reduce_buf(bt, need)) != ED_OK) goto cleanup;
      if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        capture = false;  // run this sweep directly
      } else {
        capturing = true;
      }
    }
    for (int j = k; j < m; ++j) {
      const double* res_hv = nullptr;
      if ((rc = batch_hv(bt, A, dg[cur], col[j], w, true, nullptr, &st, &res_hv)) != ED_OK) goto cleanup;
      bt->nhv++;
      const bool three = j > k && j > 0;
      k_bx_local<<<(A + 255) / 256, 256, 0, ctx->stream>>>(res_hv, A, j, m + 1, three ? 1 : 0, st,
                                                           d_coef + (size_t)64 * A);
      ctx->kernels++;
      std::vector<const double*> vs(col.begin(), col.begin() + j + 1);
      BCols vc;
      memset(&vc, 0, sizeof(vc));
      for (int i = 0; i <= j; ++i) vc.p[i] = col[i];
      const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(dim / 64 + 1, (int64_t)ctx->num_sms * 4));
      {
        // room for the dots' and the update's partials at once, so that no
        // call below moves the reduce buffer while res_upd points into it
        const size_t nd = (size_t)(j + 1) * A;
        const size_t need = std::max((nd + A) * nblk + nd, (size_t)2 * A * nblk + 2 * (size_t)A);
        if ((rc = batch_reduce_buf(bt, need)) != ED_OK) goto cleanup;
      }
      double* res_upd = bt->d_red + (size_t)2 * A * nblk;
      // first pass: the local step, the dots, the update; the second (DGKS
      // refinement) runs where the device found a realisation that needs it
      for (int pass = 0; pass < 2; ++pass) {
        const int* pred = pass ? st.again : nullptr;
        if ((rc = batch_dots_dev(bt, A, vs, w, d_coef, pass == 0 ? col[j] : nullptr,
                                 pass == 0 && three ? col[j - 1] : nullptr, d_coef + (size_t)64 * A, pred)) != ED_OK)
          goto cleanup;
        if (j + 1 <= BU_REG)
          k_batch_update_norm<true><<<nblk, 256, 0, ctx->stream>>>(vc, j + 1, d_coef, w, dim, A, bt->d_red, nblk,
                                                                   pred);
        else
          k_batch_update_norm<false><<<nblk, 256, 0, ctx->stream>>>(vc, j + 1, d_coef, w, dim, A, bt->d_red, nblk,
                                                                    pred);
        ctx->kernels++;
        k_batch_reduce<<<grid_n(ctx, (int64_t)A * 64, 8), 256, 0, ctx->stream>>>(bt->d_red, nblk, 2 * (int64_t)A,
                                                                                  res_upd, A, pred);
        ctx->kernels++;
        k_bx_post<<<(A + 255) / 256, 256, 0, ctx->stream>>>(res_upd, d_coef, A, j, m + 1, pass == 0 ? 1 : 0, st,
                                                            pred);
        ctx->kernels++;
      }
      // normalise into col[j+1] with its fixed-point copy for the next H.v
      // in the same pass (the largest exponent of the scaled block from the
      // per-realisation maxima; where it is not determined, scale only)
      k_bx_scale<<<1, 256, 0, ctx->stream>>>(A, j, m + 1, st, d_coef);
      ctx->kernels++;
      k_bx_scale_quantize<<<grid_n(ctx, colA), 256, 0, ctx->stream>>>(w, col[j + 1], d_coef, dim, A, batch_sbits(bt),
                                                                     (long long*)bt->d_xq, bt->d_gmax, st);
      ED_CHECK_LAUNCH(ctx);
    }
    if (capture) {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      capturing = false;
      cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
      if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
      if (ce == cudaSuccess) ce = cudaGraphLaunch(exec, ctx->stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      if (ce != cudaSuccess) {
        rc = ed_cuda_fail(ce, "CUDA graph of an expansion sweep", __FILE__, __LINE__);
        goto cleanup;
      }
      bt->graph_sweeps++;
    }
    {
      // alpha and beta of this sweep's steps back to the host
      const size_t na = (size_t)A * (m + 1);
      ED_CUDA(cudaMemcpyAsync(st_host.data(), st.alpha, sizeof(double) * na, cudaMemcpyDeviceToHost, ctx->stream));
      ED_CUDA(cudaMemcpyAsync(st_host.data() + na, st.beta, sizeof(double) * na, cudaMemcpyDeviceToHost,
                              ctx->stream));
      ED_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int b = 0; b < A; ++b)
        for (int jj = k; jj < m; ++jj) {
          alpha[(size_t)b * (m + 1) + jj] = st_host[(size_t)b * (m + 1) + jj];
          beta[(size_t)b * (m + 1) + jj] = st_host[(size_t)A * (m + 1) + (size_t)b * (m + 1) + jj];
        }
    }
    // projected problems, convergence and restart, per active realisation
    // (independent small eigenproblems: one host thread each)
    std::vector<int> conv_slots, keep_slots, is_conv(A, 0);
    Yall.assign((size_t)A * m * l_keep, 0.0);
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < A; ++b) {
      std::vector<double> Tb((size_t)m * m, 0.0), thb, Yb;
      const double* al = &alpha[(size_t)b * (m + 1)];
      const double* be = &beta[(size_t)b * (m + 1)];
      const double* ar = &arrow[(size_t)b * (m + 1)];
      for (int i = 0; i < k; ++i) {
        Tb[(size_t)i * m + i] = al[i];
        Tb[(size_t)i * m + k] = Tb[(size_t)k * m + i] = ar[i];
      }
      for (int jj = k; jj < m; ++jj) {
        Tb[(size_t)jj * m + jj] = al[jj];
        if (jj + 1 < m) Tb[(size_t)jj * m + jj + 1] = Tb[(size_t)(jj + 1) * m + jj] = be[jj];
      }
      ed_jacobi_eig(m, Tb, thb, Yb);
      const double bm = be[m - 1];
      int nc = 0;
      for (int i = 0; i < m; ++i) {
        const double res = std::fabs(bm * Yb[(size_t)(m - 1) * m + i]);
        if (res / std::max(std::fabs(thb[i]), 1e-300) < tol) ++nc; else break;
      }
      for (int i = 0; i < m; ++i)
        for (int c = 0; c < l_keep; ++c) Yall[((size_t)b * m + i) * l_keep + c] = Yb[(size_t)i * m + c];
      const int o = act[b];
      nconv[o] = nc;
      for (int i = 0; i < nev; ++i) bt->evals[(size_t)o * nev + i] = thb[i];
      is_conv[b] = (nc >= nev || its >= max_it) ? 1 : 0;
      // kept Ritz values and arrow couplings for the next cycle
      for (int i = 0; i < l_keep; ++i) {
        alpha[(size_t)b * (m + 1) + i] = thb[i];
        arrow[(size_t)b * (m + 1) + i] = bm * Yb[(size_t)(m - 1) * m + i];
      }
    }
    for (int b = 0; b < A; ++b) (is_conv[b] ? conv_slots : keep_slots).push_back(b);
    // restart: new columns 0..l-1 = V Y_b[:, 0..l-1]
    std::vector<double*> outc(freel.begin(), freel.begin() + l_keep);
    {
      // float-pair products only on request: the default keeps every
      // product at FP64 or better
      const bool pair = bt->restart_arith == ED_RESTART_PAIR;
      if (pair) {
        // pageable source: staged by the time cudaMemcpyAsync returns
        std::vector<float2> Yp(Yall.size());
        for (size_t q = 0; q < Yall.size(); ++q) Yp[q] = ed_host_pair(Yall[q]);
        ED_CUDA(cudaMemcpyAsync(dY, Yp.data(), sizeof(float2) * Yp.size(), cudaMemcpyHostToDevice, ctx->stream));
      } else {
        ED_CUDA(cudaMemcpyAsync(dY, Yall.data(), sizeof(double) * Yall.size(), cudaMemcpyHostToDevice, ctx->stream));
      }
      BCols vin, vout;
      memset(&vin, 0, sizeof(vin));
      memset(&vout, 0, sizeof(vout));
      for (int i = 0; i < m; ++i) vin.p[i] = col[i];
      for (int c = 0; c < l_keep; ++c) vout.p[c] = outc[c];
      int TB = 1;
      while (TB < 32 && TB < A) TB *= 2;
      const int tiles = (A + TB - 1) / TB;
      const int rows_y = (int)std::max<int64_t>(
          1, std::min<int64_t>((dim + 256 / TB - 1) / (256 / TB), ((int64_t)ctx->num_sms * 4 + tiles - 1) / tiles));
      const size_t smem = sizeof(double) * (size_t)TB * (m * 8 + 1);  // <= 127 KB (m <= 62)
      if (smem > 48 * 1024) {
        ED_CUDA(cudaFuncSetAttribute(k_batch_restart<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ED_CUDA(cudaFuncSetAttribute(k_batch_restart<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      }
      for (int c0 = 0; c0 < l_keep; c0 += 8) {
        const dim3 grid(tiles, rows_y);
        if (pair)
          k_batch_restart<true><<<grid, 256, smem, ctx->stream>>>(vin, m, dY, l_keep, vout, c0, std::min(8, l_keep - c0),
                                                                  dim, A, TB);
        else
          k_batch_restart<false><<<grid, 256, smem, ctx->stream>>>(vin, m, dY, l_keep, vout, c0, std::min(8, l_keep - c0),
                                                                   dim, A, TB);
        ED_CUDA(cudaGetLastError());
        ctx->kernels++;
      }
    }
    // converged realisations: save their Ritz vectors
    if (!conv_slots.empty()) {
      const int ns = (int)conv_slots.size();
      std::vector<int> idx(2 * (size_t)ns);
      for (int t = 0; t < ns; ++t) { idx[t] = conv_slots[t]; idx[(size_t)ns + t] = act[conv_slots[t]]; }
      ED_CUDA(cudaMemcpyAsync(d_idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, ctx->stream));
      for (int i = 0; i < nev; ++i) {
        k_batch_save<<<grid_n(ctx, dim * (int64_t)ns), 256, 0, ctx->stream>>>(outc[i], bt->d_vecs + (size_t)i * colB,
                                                                              dim, A, B, d_idx, d_idx + ns, ns);
        ctx->kernels++;
      }
    }
    // new column order: restarted vectors, then the residual vector
    std::vector<double*> newcol(m + 1, nullptr);
    for (int c = 0; c < l_keep; ++c) newcol[c] = outc[c];
    newcol[l_keep] = col[m];
    std::vector<double*> nf(freel.begin() + l_keep, freel.end());
    for (int c = 0; c < m; ++c) nf.push_back(col[c]);
    // pack the live columns and the diagonals to the realisations still active
    const int A2 = (int)keep_slots.size();
    if (A2 > 0 && A2 < A) {
      ED_CUDA(cudaMemcpyAsync(d_idx, keep_slots.data(), sizeof(int) * A2, cudaMemcpyHostToDevice, ctx->stream));
      for (int c = 0; c <= l_keep; ++c) {
        double* dst = nf.back();
        nf.pop_back();
        k_batch_pack<double><<<grid_n(ctx, dim * (int64_t)A2), 256, 0, ctx->stream>>>(newcol[c], dst, dim, A, A2,
                                                                                      d_idx);
        ctx->kernels++;
        nf.push_back(newcol[c]);
        newcol[c] = dst;
      }
      k_batch_pack<double><<<grid_n(ctx, dim * (int64_t)A2), 256, 0, ctx->stream>>>(dg[cur], dg[1 - cur], dim, A, A2,
                                                                                   d_idx);
      ctx->kernels++;
      cur = 1 - cur;
      // the fixed-point copy was made for the unpacked block
      ED_CUDA(cudaMemsetAsync(st.xq_valid, 0, sizeof(int), ctx->stream));
      std::vector<double> a2((size_t)A2 * (m + 1)), b2((size_t)A2 * (m + 1)), r2((size_t)A2 * (m + 1));
      std::vector<int> act2(A2);
      for (int t = 0; t < A2; ++t) {
        const int sl = keep_slots[t];
        act2[t] = act[sl];
        for (int i = 0; i <= m; ++i) {
          a2[(size_t)t * (m + 1) + i] = alpha[(size_t)sl * (m + 1) + i];
          b2[(size_t)t * (m + 1) + i] = beta[(size_t)sl * (m + 1) + i];
          r2[(size_t)t * (m + 1) + i] = arrow[(size_t)sl * (m + 1) + i];
        }
      }
      std::copy(a2.begin(), a2.end(), alpha.begin());
      std::copy(b2.begin(), b2.end(), beta.begin());
      std::copy(r2.begin(), r2.end(), arrow.begin());
      act.swap(act2);
    } else if (A2 == 0) {
      act.clear();
    }
    for (int c = l_keep + 1; c <= m; ++c) { newcol[c] = nf.back(); nf.pop_back(); }
    col.swap(newcol);
    freel.swap(nf);
    // the host index lists above are reused by the next cycle's copies
    ED_CUDA(cudaStreamSynchronize(ctx->stream));
    A = A2;
    k = l_keep;
  }
  // true relative residuals ||H x - theta x|| / |theta| of the saved vectors
  for (int i = 0; i < nev; ++i) {
    double* xv = bt->d_vecs + (size_t)i * colB;
    if ((rc = batch_hv(bt, B, bt->d_diag, xv, w, true)) != ED_OK) goto cleanup;
    std::vector<double> hc(B);
    for (int b = 0; b < B; ++b) hc[b] = bt->evals[(size_t)b * nev + i];
    cudaMemcpyAsync(d_coef, hc.data(), sizeof(double) * B, cudaMemcpyHostToDevice, ctx->stream);
    BCols vc;
    memset(&vc, 0, sizeof(vc));
    vc.p[0] = xv;
    k_batch_update<<<grid_n(ctx, (int64_t)colB), 256, 0, ctx->stream>>>(vc, 1, d_coef, w, dim, B);
    ctx->kernels++;
    std::vector<const double*> none;
    if ((rc = batch_dots(bt, B, none, w, true, out)) != ED_OK) goto cleanup;
    std::vector<double> r2(out.begin(), out.begin() + B);
    if ((rc = batch_dots(bt, B, none, xv, true, out)) != ED_OK) goto cleanup;
    for (int b = 0; b < B; ++b)
      bt->errs[(size_t)b * nev + i] =
          std::sqrt(r2[b]) / std::max(std::fabs(bt->evals[(size_t)b * nev + i]) * std::sqrt(out[b]), 1e-300);
  }
  bt->nev = nev;
  bt->nrep = nev;
  bt->its = its;
  bt->nconv = nconv;
  for (int b = 0; b < B; ++b) {
    nconv_host[b] = nconv[b];
    for (int i = 0; i < nev; ++i) {
      evals_host[(size_t)b * nev + i] = bt->evals[(size_t)b * nev + i];
      errs_host[(size_t)b * nev + i] = bt->errs[(size_t)b * nev + i];
    }
  }
cleanup:
  if (capturing) {  // an error inside a captured sweep: close the capture
    cudaGraph_t graph = nullptr;
    cudaStreamEndCapture(ctx->stream, &graph);
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
  }
  cudaStreamSynchronize(ctx->stream);
  cudaFree(st_buf);
  cudaFree(st_int);
  cudaFree(pool);
  cudaFree(w);
  cudaFree(dg[0]);
  cudaFree(dg[1]);
  cudaFree(d_coef);
  cudaFree(d_idx);
  cudaFree(dY);
  return rc;
}

int ed_batch_solve_many(ed_batch* const* bts, int count, int nev, int ncv, double tol, int max_it, uint64_t seed,
                        double* const* evals_host, double* const* errs_host, int* const* nconv_host) {
  if (!bts || count < 1 || !evals_host || !errs_host || !nconv_host) return ed_fail(ED_EINVAL, "null argument");
  for (int i = 0; i < count; ++i) {
    if (!bts[i] || !evals_host[i] || !errs_host[i] || !nconv_host[i]) return ed_fail(ED_EINVAL, "null argument");
    for (int j = 0; j < i; ++j)
      if (bts[j]->h->ctx == bts[i]->h->ctx)
        return ed_fail(ED_EINVAL, "each batch of ed_batch_solve_many needs its own environment (stream)");
  }
  // one host thread per batch; every batch issues to its own context's
  // stream, so the device overlaps them (the gathers of one sector's H.v on
  // the L1 path beside another's FP64-bound Gram-Schmidt)
  std::vector<int> rc(count, ED_OK);
  std::vector<std::string> msg(count);
  auto run = [&](int i) {
    ed_batch* bt = bts[i];
    if (cudaSetDevice(bt->h->ctx->device) != cudaSuccess) {
      rc[i] = ed_cuda_fail(cudaGetLastError(), "cudaSetDevice", __FILE__, __LINE__);
    } else {
      rc[i] = ed_batch_solve(bt, nev, ncv, tol, max_it, seed, evals_host[i], errs_host[i], nconv_host[i]);
    }
    if (rc[i] != ED_OK) {
      char buf[512];
      ed_last_error(buf, sizeof(buf));
      msg[i] = buf;
    }
  };
  std::vector<std::thread> th;
  for (int i = 1; i < count; ++i) th.emplace_back(run, i);
  run(0);
  for (auto& t : th) t.join();
  for (int i = 0; i < count; ++i)
    if (rc[i] != ED_OK) return ed_fail(rc[i], "batch " + std::to_string(i) + ": " + msg[i]);
  return ED_OK;
}

int ed_batch_get_eigenvector(ed_batch* bt, int b, int i, ed_cplx* vec_dev) {
  if (!bt || !vec_dev) return ed_fail(ED_EINVAL, "null argument");
  if (!bt->d_vecs || i < 0 || i >= bt->nrep || b < 0 || b >= bt->B) return ed_fail(ED_EINVAL, "index out of range");
  ed_ctx* ctx = bt->h->ctx;
  k_batch_extract<<<grid_n(ctx, bt->dim), 256, 0, ctx->stream>>>(bt->d_vecs + (size_t)i * bt->dim * bt->B, bt->dim,
                                                                bt->B, b, (double2*)vec_dev);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

int ed_batch_set_graphs(ed_batch* bt, int on) {
  if (!bt) return ed_fail(ED_EINVAL, "null batch");
  bt->graphs = on != 0;
  return ED_OK;
}

int ed_batch_graph_sweeps(const ed_batch* bt, int64_t* n) {
  if (!bt || !n) return ed_fail(ED_EINVAL, "null argument");
  *n = bt->graph_sweeps;
  return ED_OK;
}

int ed_batch_set_hv_tile(ed_batch* bt, int rows, int threads) {
  if (!bt) return ed_fail(ED_EINVAL, "null batch");
  if (rows == 0 && threads == 0) {
    bt->hv_variant = -1;
    bt->hv_forced = false;
    return ED_OK;
  }
  for (int v = 0; v < kBhVariants; ++v)
    if (kBhRows[v / 2] == rows && kBhThreads[v % 2] == threads) {
      bt->hv_variant = v;
      bt->hv_forced = true;
      return ED_OK;
    }
  return ed_fail(ED_EINVAL, "unknown batched H.v tile (rows 4/8/16/32, threads 128/256)");
}

int ed_batch_hv_tile(const ed_batch* bt, int* rows, int* threads) {
  if (!bt || !rows || !threads) return ed_fail(ED_EINVAL, "null argument");
  *rows = bt->hv_variant < 0 ? 0 : kBhRows[bt->hv_variant / 2];
  *threads = bt->hv_variant < 0 ? 0 : kBhThreads[bt->hv_variant % 2];
  return ED_OK;
}

int ed_batch_set_restart_arithmetic(ed_batch* bt, int mode) {
  if (!bt) return ed_fail(ED_EINVAL, "null batch");
  if (mode != ED_RESTART_AUTO && mode != ED_RESTART_FP64 && mode != ED_RESTART_PAIR)
    return ed_fail(ED_EINVAL, "unknown restart arithmetic");
  bt->restart_arith = mode;
  return ED_OK;
}

int ed_batch_stats(ed_batch* bt, int* its, int64_t* n_hv) {
  if (!bt) return ed_fail(ED_EINVAL, "null batch");
  if (its) *its = bt->its;
  if (n_hv) *n_hv = bt->nhv;
  return ED_OK;
}

}  // extern "C"
