// Device helpers: chunked combinadic rank, start-vector hash.
#pragma once
#include <cstdint>
#include "ed_internal.h"

// Rank of a state with nup set bits, tables in shared (or global) memory.
// K is the number of chunks (compile-time).
template <int K>
__device__ __forceinline__ uint32_t ed_rank(uint32_t s, const uint32_t* __restrict__ tab, const RankTables& rt) {
  if (K == 1) return tab[s];
  uint32_t r = 0;
  int c = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    uint32_t chunk = (s >> rt.off[k]) & ((1u << rt.w[k]) - 1u);
    if (k == 0) {
      r += tab[chunk];
    } else if (k == K - 1) {
      r += tab[rt.base[k] + chunk];
    } else {
      r += tab[rt.base[k] + (c << rt.w[k]) + chunk];
    }
    c += __popc(chunk);
  }
  return r;
}

// Per-row rank state for incremental ranks of bond-flipped states: chunk
// values, set bits below each chunk, and each chunk's table entry.
template <int K>
struct RowRank {
  uint32_t cv[K];
  int pc[K];
  uint32_t tv[K];
};

template <int K>
__device__ __forceinline__ uint32_t ed_tab_index(const RankTables& rt, int k, int p, uint32_t c) {
  if (k == 0) return c;
  if (k == K - 1) return (uint32_t)rt.base[k] + c;
  return (uint32_t)rt.base[k] + ((uint32_t)p << rt.w[k]) + c;
}

template <int K>
__device__ __forceinline__ void ed_row_rank(uint32_t s, const uint32_t* __restrict__ tab, const RankTables& rt,
                                            RowRank<K>& R) {
  int c = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    R.cv[k] = (s >> rt.off[k]) & ((1u << rt.w[k]) - 1u);
    R.pc[k] = c;
    R.tv[k] = tab[ed_tab_index<K>(rt, k, c, R.cv[k])];
    c += __popc(R.cv[k]);
  }
}

// Rank of the state with bond b flipped, from the unflipped state's rank r:
// only chunks ci..cj change (the bond is antiparallel: exactly one of its
// bits is set, so the set-bit count above chunk cj is unchanged).
template <int K>
__device__ __forceinline__ uint32_t ed_rank_flip(uint32_t r, uint32_t s, const uint32_t* __restrict__ tab,
                                                 const RankTables& rt, const RowRank<K>& R, const BondSet& bs, int b) {
  const int ci = bs.ci[b], cj = bs.cj[b];
  const int d = ((s >> bs.lo[b]) & 1u) ? -1 : 1;
  uint32_t rr = r;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (k >= ci && k <= cj) {
      const uint32_t c = R.cv[k] ^ (uint32_t)bs.xm[b][k];
      const int p = R.pc[k] + (k > ci ? d : 0);
      rr += tab[ed_tab_index<K>(rt, k, p, c)] - R.tv[k];
    }
  }
  return rr;
}

// Counter-based splitmix64 (deterministic, identical on host and device).
__device__ __forceinline__ uint64_t ed_splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Block reduction of NV doubles (fixed tree order); thread 0 ends with the
// block sums in v[].  sh holds NV * 32 doubles.
template <int NV>
__device__ __forceinline__ void ed_block_reduce(double (&v)[NV], double* sh) {
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

// Running max of the high 32 bits of |v| (sign, exponent and the top 20
// fraction bits; for non-negative doubles their order is that of the
// integers): two integer instructions per value, since FP64 min/max issue on
// GB300's slow FP64 unit and a 64-bit compare costs more.  The result, as the
// double whose low word is zero, is a lower bound of max |v| with the same
// high 32 bits.
__device__ __forceinline__ unsigned int ed_absmax_hi(unsigned int m, double v) {
  return max(m, (unsigned int)(__double_as_longlong(v) >> 32) & 0x7FFFFFFFu);
}

__device__ __forceinline__ double ed_absmax_hi_value(unsigned int m) {
  return __longlong_as_double((long long)((unsigned long long)m << 32));
}

// Block maximum of v (>= 0) into thread 0's v; sh holds 32 doubles.
__device__ __forceinline__ void ed_block_max(double& v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < nw ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  }
}

// Load the rank tables into shared memory (block-cooperative).
__device__ __forceinline__ void ed_load_tables(uint32_t* stab, const RankTables& rt) {
  for (int i = threadIdx.x; i < rt.total; i += blockDim.x) stab[i] = rt.tab[i];
  __syncthreads();
}

// Float pairs: an FP64 value v read as hi + lo (two floats) so that products
// can be formed on the FP32 units.  hi = the leading 24 significand bits of v
// (truncated), lo = the next 23 (rounded): |v - hi - lo| <= 2^-47 |v|.  Built
// with integer operations on the bits only.  |v| < 2^-126 gives 0 (below
// 2^-103 lo is 0); |v| >= 2^128 and non-finite v give NaN.
__device__ __forceinline__ float2 ed_pair(double v) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const unsigned int hw = (unsigned int)(bits >> 32), lw = (unsigned int)bits;
  const unsigned int sign = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7FFu);
  // hi: float exponent e - 1023 + 127 (the 9-bit field wraps correctly in
  // range), fraction = the top 23 fraction bits of v
  unsigned int hb = ((__funnelshift_l(lw, hw, 3) - (896u << 23)) & 0x7FFFFFFFu) | sign;
  // lo: fraction bits 28..6 rounded at bit 5, as (2^E + m ulp) - 2^E exactly
  // (a carry out of m moves into the exponent, which is the right value)
  const unsigned int m = (((lw & 0x1FFFFFFFu) >> 5) + 1u) >> 1;
  const unsigned int base = (unsigned int)(e - 919) << 23;
  float lo = __fsub_rn(__uint_as_float(base + m), __uint_as_float(base));
  lo = __uint_as_float(__float_as_uint(lo) | sign);
  if ((unsigned int)(e - 897) > 253u) hb = e > 1150 ? 0x7FC00000u : sign;
  if ((unsigned int)(e - 920) > 230u) lo = 0.0f;
  return make_float2(__uint_as_float(hb), lo);
}

// (s, c) += a * b for float pairs a, b: the product exact to first order (hi*hi
// exactly with an FMA, the other three terms added; error below 2^-45 |a b|
// with the splitting), summed into the pair (s, c) by Knuth's TwoSum.
__device__ __forceinline__ void ed_pair_mac(float2 a, float2 b, float& s, float& c) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  e = __fmaf_rn(a.y, b.y, e);
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  c = __fadd_rn(c, __fadd_rn(err, e));
  s = t;
}

__device__ __forceinline__ double ed_pair_value(float s, float c) { return (double)s + (double)c; }

// The same split on the host, rounding twice: error below 2^-48 |v| (|v| < 2^127).
static inline float2 ed_host_pair(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

// 128-bit signed T times 2^X, rounded to nearest even, as an FP64 value,
// with integer operations only.  Results below 2^-1022 flush to zero.
__device__ __forceinline__ double ed_fx128_to_double(long long hi, unsigned long long lo, int X) {
  const bool neg = hi < 0;
  if (neg) {
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ll : 0ll);
  }
  const unsigned long long uh = (unsigned long long)hi;
  if (uh == 0ull && lo == 0ull) return 0.0;
  const int L = uh ? 128 - __clzll((long long)uh) : 64 - __clzll((long long)lo);  // bit length
  unsigned long long m;
  int bexp = X + L + 1022;
  if (L <= 53) {
    m = lo << (53 - L);
  } else {
    const int sr = L - 53;  // 1 .. 75
    unsigned long long rem, half;
    if (sr < 64) {
      m = (lo >> sr) | (sr ? (uh << (64 - sr)) : 0ull);
      rem = lo & ((1ull << sr) - 1ull);
      half = 1ull << (sr - 1);
      const bool up = rem > half || (rem == half && (m & 1ull));
      m += up ? 1ull : 0ull;
    } else {
      const int s2 = sr - 64;
      m = uh >> s2;
      const unsigned long long remh = uh & ((s2 ? (1ull << s2) : 1ull) - 1ull);
      const bool gt = s2 ? (remh > (1ull << (s2 - 1)) || (remh == (1ull << (s2 - 1)) && lo != 0ull)) : (lo > (1ull << 63));
      const bool eq = s2 ? (remh == (1ull << (s2 - 1)) && lo == 0ull) : (lo == (1ull << 63));
      m += (gt || (eq && (m & 1ull))) ? 1ull : 0ull;
    }
    if (m >> 53) {
      m >>= 1;
      ++bexp;
    }
  }
  if (bexp <= 0) return 0.0;
  const unsigned long long bits =
      ((unsigned long long)neg << 63) | ((unsigned long long)bexp << 52) | (m & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}
