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

// Load the rank tables into shared memory (block-cooperative).
__device__ __forceinline__ void ed_load_tables(uint32_t* stab, const RankTables& rt) {
  for (int i = threadIdx.x; i < rt.total; i += blockDim.x) stab[i] = rt.tab[i];
  __syncthreads();
}
