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

// Counter-based splitmix64 (deterministic, identical on host and device).
__device__ __forceinline__ uint64_t ed_splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Load the rank tables into shared memory (block-cooperative).
__device__ __forceinline__ void ed_load_tables(uint32_t* stab, const RankTables& rt) {
  for (int i = threadIdx.x; i < rt.total; i += blockDim.x) stab[i] = rt.tab[i];
  __syncthreads();
}
