// Fixed-Sz basis on the device: Basis(env, total_mag) (src/basis.cpp:56-94),
// BasisHelper::search_elem (src/basis.cpp:9-36) and
// HamiltHelper::search_index (src/hamiltonian.cpp:9-27).
//
// The reference enumerates a rank's states with Gosper's hack from an
// unranked first element; here every state is unranked independently (one
// thread per index, exact integer binomials), which yields the same
// ascending sequence without a serial dependency.
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>

__constant__ uint32_t c_binom[ED_MAX_SPINS + 1][ED_MAX_SPINS + 1];
static bool g_binom_uploaded[64] = {false};

uint64_t ed_binom(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  static uint64_t T[65][65];
  static bool ready = false;
  if (!ready) {
    for (int a = 0; a <= 64; ++a) {
      T[a][0] = 1;
      for (int b = 1; b <= 64; ++b) T[a][b] = a == 0 ? 0 : T[a - 1][b - 1] + T[a - 1][b];
    }
    ready = true;
  }
  return T[n][k];
}

static int upload_binom(int device) {
  if (device >= 0 && device < 64 && g_binom_uploaded[device]) return ED_OK;
  uint32_t h[ED_MAX_SPINS + 1][ED_MAX_SPINS + 1];
  for (int n = 0; n <= ED_MAX_SPINS; ++n)
    for (int k = 0; k <= ED_MAX_SPINS; ++k) {
      uint64_t v = ed_binom(n, k);
      h[n][k] = v > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)v;  // only C(32,k) can exceed; never used as a bound
    }
  ED_CUDA(cudaMemcpyToSymbol(c_binom, h, sizeof(h)));
  if (device >= 0 && device < 64) g_binom_uploaded[device] = true;
  return ED_OK;
}

// Chunk layout: the smallest K whose tables fit in 56 KB of shared memory.
int ed_build_rank_tables(int N, int nup, RankTables& rt, std::vector<uint32_t>& tab) {
  const int kMaxEntries = 14336;
  int K = 0;
  int w[ED_RANK_MAX_CHUNKS] = {0}, off[ED_RANK_MAX_CHUNKS] = {0}, base[ED_RANK_MAX_CHUNKS] = {0};
  int total = 0;
  for (int k = 1; k <= ED_RANK_MAX_CHUNKS; ++k) {
    int b = N / k, rem = N % k, o = 0, t = 0;
    for (int c = 0; c < k; ++c) {
      w[c] = b + (c < rem ? 1 : 0);
      off[c] = o;
      o += w[c];
    }
    for (int c = 0; c < k; ++c) {
      base[c] = t;
      if (k == 1 || c == 0 || c == k - 1) t += 1 << w[c];
      else t += (off[c] + 1) << w[c];
    }
    if (t <= kMaxEntries || k == ED_RANK_MAX_CHUNKS) { K = k; total = t; break; }
  }
  tab.assign(total, 0u);
  for (int c = 0; c < K; ++c) {
    int nb = 1 << w[c];
    int crange = (K == 1 || c == 0 || c == K - 1) ? 1 : off[c] + 1;
    for (int cc = 0; cc < crange; ++cc)
      for (int bits = 0; bits < nb; ++bits) {
        int below;
        if (c == 0) below = 0;
        else if (c == K - 1) below = nup - __builtin_popcount((unsigned)bits);
        else below = cc;
        uint64_t v = 0;
        if (below >= 0 && below <= off[c]) {
          int t = 0;
          for (int q = 0; q < w[c]; ++q)
            if ((bits >> q) & 1) { ++t; v += ed_binom(off[c] + q, below + t); }
        }
        size_t idx = (size_t)base[c] + (size_t)cc * nb + bits;
        tab[idx] = (uint32_t)v;
      }
  }
  rt.K = K; rt.nup = nup; rt.total = total; rt.tab = nullptr;
  for (int c = 0; c < ED_RANK_MAX_CHUNKS; ++c) { rt.w[c] = w[c]; rt.off[c] = off[c]; rt.base[c] = base[c]; }
  return ED_OK;
}

// Unrank index -> state (greedy from the top bit, basis.cpp:9-36).
__device__ __forceinline__ uint32_t ed_unrank(uint64_t index, int N, int nup) {
  uint64_t rest = index;
  uint32_t elem = 0;
  int sup = nup;
  for (int pi = N - 1; pi >= 0 && sup > 0; --pi) {
    uint64_t b = (pi < sup) ? 0 : c_binom[pi][sup];
    if (b <= rest) {
      rest -= b;
      elem |= 1u << pi;
      --sup;
    }
  }
  return elem;
}

__global__ void k_basis_states(int N, int nup, int64_t dim, uint32_t* __restrict__ states) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += stride)
    states[i] = ed_unrank((uint64_t)i, N, nup);
}

__global__ void k_unrank(int N, int nup, const int64_t* __restrict__ ranks, int64_t n, uint32_t* __restrict__ out) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = ed_unrank((uint64_t)ranks[i], N, nup);
}

template <int K>
__global__ void k_rank(RankTables rt, const uint32_t* __restrict__ states, int64_t n, int64_t* __restrict__ out) {
  extern __shared__ uint32_t stab[];
  ed_load_tables(stab, rt);
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = (int64_t)ed_rank<K>(states[i], stab, rt);
}

static int grid_for(ed_ctx* ctx, int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  int64_t cap = (int64_t)ctx->num_sms * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int ed_launch_basis_states(ed_ctx* ctx, int N, int nup, int64_t dim, uint32_t* states) {
  ED_TRY(upload_binom(ctx->device));
  k_basis_states<<<grid_for(ctx, dim, 256), 256, 0, ctx->stream>>>(N, nup, dim, states);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

int ed_launch_unrank(ed_ctx* ctx, const ed_basis* b, const int64_t* ranks_dev, int64_t n, uint32_t* states_dev) {
  ED_TRY(upload_binom(ctx->device));
  k_unrank<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(b->nspins, b->nup, ranks_dev, n, states_dev);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

template <int K>
static int launch_rank_k(ed_ctx* ctx, const ed_basis* b, const uint32_t* s, int64_t n, int64_t* out) {
  size_t smem = (size_t)b->rt.total * sizeof(uint32_t);
  ED_CUDA(cudaFuncSetAttribute(k_rank<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_rank<K><<<grid_for(ctx, n, 256), 256, smem, ctx->stream>>>(b->rt, s, n, out);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

int ed_launch_rank(ed_ctx* ctx, const ed_basis* b, const uint32_t* states_dev, int64_t n, int64_t* ranks_dev) {
  switch (b->rt.K) {
    case 1: return launch_rank_k<1>(ctx, b, states_dev, n, ranks_dev);
    case 2: return launch_rank_k<2>(ctx, b, states_dev, n, ranks_dev);
    case 3: return launch_rank_k<3>(ctx, b, states_dev, n, ranks_dev);
    default: return launch_rank_k<4>(ctx, b, states_dev, n, ranks_dev);
  }
}
