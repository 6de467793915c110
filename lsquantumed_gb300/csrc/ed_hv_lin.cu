// Fixed-point matrix-free H.v with a two-table (low/high half) combinadic rank.
//
// The basis state s splits into c0 = the low w0 bits and c1 = the high
// w1 = N - w0 bits.  With p_i the position of the i-th set bit (ascending),
// the rank of s in the fixed-Sz basis (ascending integers, the order of
// Basis::generate_int_basis, basis.cpp:192-215) is sum_i C(p_i, i), which
// splits into T0[c0] + T1[c1]: the set-bit count below the high half is
// nup - popc(c1), so the high half's share depends on c1 alone.  T0 (< 2^16
// per entry for w0 <= 14) sits in shared memory as uint16, T1 in global
// memory behind the read-only cache (consecutive rows share c1).
//
// A bond flip then costs one table entry: bonds inside the low half change
// only T0 (target rank r - T0[c0] + T0[c0 ^ m0]), bonds inside the high half
// only T1 (target r - T1[c1] + T1[c1 ^ m1], the same low offset in another
// block: consecutive rows gather consecutive entries), and bonds across the
// halves both.  The gathered terms are int64 fixed-point copies of x (see
// k_quantize64) summed exactly per coupling type, so the result is
// bit-identical to every other fixed-point kernel of this library.
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#define LIN_MAX_W0 14

// Bond words by class (0 = low half, 1 = high half, 2 = across) and coupling
// type: lo 32 bits = mask within the low half, hi 32 = mask within the high
// half (shifted down by w0).
struct LinSegs {
  int w0;
  int seg[7];
  unsigned long long word[ED_MAX_BONDS];
};

struct ed_lin {
  LinSegs segs{};
  int built_nb = -1;
  int variant[4] = {-1, -1, -1, -1};  // launch variants [2 * dot + real storage] chosen by lin_autotune; -1: not yet
  // per-bond couplings: J_b / 2 of each word as fixed point, value = c * 2^pbexp
  bool per_bond = false;
  std::vector<long long> coef;
  long long* d_coef = nullptr;  // device copy of coef (ED_MAX_BONDS entries)
  int pbexp = 0;
  ~ed_lin() {
    if (d_coef) cudaFree(d_coef);
  }
};

static uint64_t binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (uint64_t)(n - k + i) / (uint64_t)i;
  return r;
}

void ed_lin_free(ed_lin* L) { delete L; }

int ed_basis_lin_tables(ed_basis* b) {
  const int N = b->nspins, nup = b->nup;
  const int w0 = std::min(LIN_MAX_W0, (N + 1) / 2), w1 = N - w0;
  std::vector<uint16_t> t0((size_t)1 << w0);
  std::vector<uint32_t> t1((size_t)1 << w1);
  for (uint32_t c = 0; c < t0.size(); ++c) {
    uint64_t v = 0;
    int k = 0;
    for (int p = 0; p < w0; ++p)
      if ((c >> p) & 1u) v += binom(p, ++k);
    t0[c] = (uint16_t)v;
  }
  for (uint32_t c = 0; c < t1.size(); ++c) {
    const int k0 = nup - __builtin_popcount(c);
    uint64_t v = 0;
    if (k0 >= 0 && k0 <= w0) {
      int k = k0;
      for (int q = 0; q < w1; ++q)
        if ((c >> q) & 1u) v += binom(w0 + q, ++k);
    }
    t1[c] = (uint32_t)v;
  }
  if (cudaMalloc(&b->d_lin_t0, t0.size() * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&b->d_lin_t1, t1.size() * sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    return ed_fail(ED_ENOMEM, "rank tables do not fit in device memory");
  }
  cudaError_t e1 = cudaMemcpy(b->d_lin_t0, t0.data(), t0.size() * sizeof(uint16_t), cudaMemcpyHostToDevice);
  cudaError_t e2 = cudaMemcpy(b->d_lin_t1, t1.data(), t1.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e1 != cudaSuccess || e2 != cudaSuccess)
    return ed_cuda_fail(e1 != cudaSuccess ? e1 : e2, "rank table upload", __FILE__, __LINE__);
  b->lin_w0 = w0;
  return ED_OK;
}

// Bond words for h (once per bond set: rebuilt after build_off_diag).
static int lin_prepare(ed_ham* h) {
  const ed_basis* b = h->basis;
  if (!h->lin) h->lin = new ed_lin();
  ed_lin* L = h->lin;
  if (L->built_nb != h->bs.nb) {
    LinSegs& sg = L->segs;
    memset(&sg, 0, sizeof(sg));
    sg.w0 = b->lin_w0;
    const uint32_t low = (1u << b->lin_w0) - 1u;
    int n = 0;
    for (int cls = 0; cls < 3; ++cls)
      for (int t = 0; t < 2; ++t) {
        sg.seg[cls * 2 + t] = n;
        for (int q = 0; q < h->bs.nb; ++q) {
          const uint32_t m = h->bs.mask[q];
          if (h->bs.type[q] != t || __builtin_popcount(m) != 2) continue;  // i == j never couples
          const uint32_t m0 = m & low, m1 = m >> b->lin_w0;
          const int c = m1 == 0 ? 0 : (m0 == 0 ? 1 : 2);
          if (c != cls) continue;
          sg.word[n++] = (unsigned long long)m0 | ((unsigned long long)m1 << 32);
        }
      }
    sg.seg[6] = n;
    L->per_bond = h->bs.per_bond != 0;
    L->coef.clear();
    if (L->per_bond) {
      // one coupling per bond: the words by class only (the second type of
      // each class stays empty), each with its J_b / 2 in fixed point.  With
      // |xq| < 2^sbits and at most nb terms, |c| < 2^kc keeps every row's
      // exact sum below 2^126.
      n = 0;
      std::vector<double> cf;
      for (int cls = 0; cls < 3; ++cls) {
        sg.seg[cls * 2] = n;
        for (int q = 0; q < h->bs.nb; ++q) {
          const uint32_t m = h->bs.mask[q];
          if (__builtin_popcount(m) != 2) continue;
          const uint32_t m0 = m & low, m1 = m >> b->lin_w0;
          const int c = m1 == 0 ? 0 : (m0 == 0 ? 1 : 2);
          if (c != cls) continue;
          sg.word[n++] = (unsigned long long)m0 | ((unsigned long long)m1 << 32);
          cf.push_back(h->bs.chalf[h->bs.type[q]]);
        }
        sg.seg[cls * 2 + 1] = n;
      }
      sg.seg[6] = n;
      double mx = 0.0;
      for (double v : cf) mx = std::max(mx, std::fabs(v));
      int e = 0;
      if (mx > 0.0) std::frexp(mx, &e);  // mx < 2^e
      int lg = 0;
      while ((1 << lg) < h->bs.nb + 1) ++lg;
      const int kc = 125 - ed_fx64_sbits(h) - lg;
      for (double v : cf) L->coef.push_back(std::llround(std::ldexp(v, kc - e)));
      L->pbexp = e - kc;
      if (!L->d_coef && cudaMalloc(&L->d_coef, sizeof(long long) * ED_MAX_BONDS) != cudaSuccess) {
        cudaGetLastError();
        L->d_coef = nullptr;
        return ed_fail(ED_ENOMEM, "per-bond coefficient table does not fit in device memory");
      }
      if (!L->coef.empty())
        ED_CUDA(cudaMemcpyAsync(L->d_coef, L->coef.data(), sizeof(long long) * L->coef.size(), cudaMemcpyHostToDevice,
                                h->ctx->stream));  // ordered after earlier launches that read it
    }
    L->built_nb = h->bs.nb;
  }
  return ED_OK;
}

// Bonds inside one half: the flipped state's rank is rb + T[c ^ m].
template <bool CHECK, bool HIGH, int U, bool RX>
__device__ __forceinline__ void lin_half(const LinSegs& sg, int b0, int b1, uint32_t c, uint32_t rb,
                                         const uint16_t* __restrict__ t0s, const uint32_t* __restrict__ t1,
                                         const longlong2* __restrict__ xq, long long& ar, long long& ai, bool& bad) {
  const long long kNaN = (long long)0x8000000000000000ull;
  for (int b = b0; b < b1; b += U) {
    uint32_t tgt[U];
    bool on[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool inb = b + u < b1;
      const unsigned long long w = inb ? sg.word[b + u] : 0ull;
      const uint32_t m = HIGH ? (uint32_t)(w >> 32) : (uint32_t)w;
      const uint32_t t = c & m;
      on[u] = t != 0u && t != m;  // m == 0 (past the end) is never on
      tgt[u] = rb + (HIGH ? __ldg(&t1[c ^ m]) : (uint32_t)t0s[c ^ m]);
    }
    if (RX) {
      const long long* xr = (const long long*)xq;
      long long q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) q[u] = on[u] ? __ldg(&xr[tgt[u]]) : 0ll;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (CHECK) bad |= q[u] == kNaN;
        ar += q[u];
      }
    } else {
      longlong2 q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) q[u] = on[u] ? __ldg(&xq[tgt[u]]) : make_longlong2(0, 0);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (CHECK) bad |= (q[u].x == kNaN) | (q[u].y == kNaN);
        ar += q[u].x;
        ai += q[u].y;
      }
    }
  }
}

// Bonds across the halves: one site in each, the rank is T0[c0 ^ m0] + T1[c1 ^ m1].
template <bool CHECK, int U, bool RX>
__device__ __forceinline__ void lin_cross(const LinSegs& sg, int b0, int b1, uint32_t c0, uint32_t c1,
                                          const uint16_t* __restrict__ t0s, const uint32_t* __restrict__ t1,
                                          const longlong2* __restrict__ xq, long long& ar, long long& ai, bool& bad) {
  const long long kNaN = (long long)0x8000000000000000ull;
  for (int b = b0; b < b1; b += U) {
    uint32_t tgt[U];
    bool on[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool inb = b + u < b1;
      const unsigned long long w = inb ? sg.word[b + u] : 0ull;
      const uint32_t m0 = (uint32_t)w, m1 = (uint32_t)(w >> 32);
      on[u] = inb && (((c0 & m0) != 0u) != ((c1 & m1) != 0u));
      tgt[u] = (uint32_t)t0s[c0 ^ m0] + __ldg(&t1[c1 ^ m1]);
    }
    if (RX) {
      const long long* xr = (const long long*)xq;
      long long q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) q[u] = on[u] ? __ldg(&xr[tgt[u]]) : 0ll;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (CHECK) bad |= q[u] == kNaN;
        ar += q[u];
      }
    } else {
      longlong2 q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) q[u] = on[u] ? __ldg(&xq[tgt[u]]) : make_longlong2(0, 0);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (CHECK) bad |= (q[u].x == kNaN) | (q[u].y == kNaN);
        ar += q[u].x;
        ai += q[u].y;
      }
    }
  }
}

// rio: x and y are real storage (double[dim]); the input is then real (RX).
template <bool CHECK, bool DOT, int U, bool RX>
__device__ __forceinline__ void lin_rows(const uint32_t* __restrict__ states, const double* __restrict__ diag,
                                         const double2* __restrict__ x, const longlong2* __restrict__ xq,
                                         double2* __restrict__ y, int64_t dim, const uint16_t* __restrict__ t0s,
                                         const uint32_t* __restrict__ t1, const LinSegs& sg, double c0c, double c1c,
                                         double s1, double s2, double (&dacc)[3], bool rio) {
  const uint32_t low = (1u << sg.w0) - 1u;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const uint32_t s = states[r];
    const uint32_t c0 = s & low, c1 = s >> sg.w0;
    const uint32_t rr = (uint32_t)r;
    const uint32_t rb0 = rr - (uint32_t)t0s[c0];
    const uint32_t rb1 = rr - __ldg(&t1[c1]);
    long long a[4] = {0, 0, 0, 0};  // nn re, nn im, nnn re, nnn im
    bool bad = false;
    lin_half<CHECK, false, U, RX>(sg, sg.seg[0], sg.seg[1], c0, rb0, t0s, t1, xq, a[0], a[1], bad);
    lin_half<CHECK, false, U, RX>(sg, sg.seg[1], sg.seg[2], c0, rb0, t0s, t1, xq, a[2], a[3], bad);
    lin_half<CHECK, true, U, RX>(sg, sg.seg[2], sg.seg[3], c1, rb1, t0s, t1, xq, a[0], a[1], bad);
    lin_half<CHECK, true, U, RX>(sg, sg.seg[3], sg.seg[4], c1, rb1, t0s, t1, xq, a[2], a[3], bad);
    lin_cross<CHECK, U, RX>(sg, sg.seg[4], sg.seg[5], c0, c1, t0s, t1, xq, a[0], a[1], bad);
    lin_cross<CHECK, U, RX>(sg, sg.seg[5], sg.seg[6], c0, c1, t0s, t1, xq, a[2], a[3], bad);
    const double d = diag[r];
    const double2 xv = rio ? make_double2(((const double*)x)[r], 0.0) : x[r];
    const double s0r = (double)a[0] * s1 * s2, s0i = (double)a[1] * s1 * s2;
    const double s1r = (double)a[2] * s1 * s2, s1i = (double)a[3] * s1 * s2;
    double yr = fma(d, xv.x, fma(c0c, s0r, c1c * s1r));
    double yi = fma(d, xv.y, fma(c0c, s0i, c1c * s1i));
    if (CHECK && bad) { yr = __longlong_as_double(0x7FF8000000000000ll); yi = yr; }
    if (rio) ((double*)y)[r] = yr;
    else y[r] = make_double2(yr, yi);
    if (DOT) {
      dacc[0] = fma(xv.x, yr, fma(xv.y, yi, dacc[0]));
      dacc[1] = fma(xv.x, yi, fma(-xv.y, yr, dacc[1]));
      dacc[2] = fma(yr, yr, fma(yi, yi, dacc[2]));
    }
  }
}

// DOT: partial[item * gridDim.x + block] for item 0/1 = Re/Im x^H y, 2 = ||y||^2.
// U: bonds per unrolled batch (gathers in flight per thread); MINB: blocks
// per SM the register allocation must allow.
template <bool DOT, int U, int MINB>
__global__ void __launch_bounds__(256, MINB) k_hv_lin(const uint32_t* __restrict__ states, const double* __restrict__ diag,
                                                const double2* __restrict__ x, const longlong2* __restrict__ xq,
                                                const int* __restrict__ gmax_p, int sbits, double2* __restrict__ y,
                                                int64_t dim, const uint16_t* __restrict__ t0,
                                                const uint32_t* __restrict__ t1, const LinSegs sg, double c0c,
                                                double c1c, double* __restrict__ partial, int rio_flag) {
  extern __shared__ uint16_t t0s[];
  const bool rio = rio_flag != 0;
  const int n0 = 1 << sg.w0;
  for (int i = threadIdx.x; i < n0; i += blockDim.x) t0s[i] = t0[i];
  __syncthreads();
  const int e_unit = gmax_p[0] - 1022 - sbits;
  const double s1 = __longlong_as_double((long long)(e_unit / 2 + 1023) << 52);
  const double s2 = __longlong_as_double((long long)(e_unit - e_unit / 2 + 1023) << 52);
  double dacc[3] = {0.0, 0.0, 0.0};
  // gmax_p[1]: some input entry is not finite (track the rows that gather it);
  // gmax_p[2] == 0: x is real and xq holds only real parts
  const bool rx = gmax_p[2] == 0;
  if (gmax_p[1]) {
    if (rx) lin_rows<true, DOT, U, true>(states, diag, x, xq, y, dim, t0s, t1, sg, c0c, c1c, s1, s2, dacc, rio);
    else lin_rows<true, DOT, U, false>(states, diag, x, xq, y, dim, t0s, t1, sg, c0c, c1c, s1, s2, dacc, rio);
  } else {
    if (rx) lin_rows<false, DOT, U, true>(states, diag, x, xq, y, dim, t0s, t1, sg, c0c, c1c, s1, s2, dacc, rio);
    else lin_rows<false, DOT, U, false>(states, diag, x, xq, y, dim, t0s, t1, sg, c0c, c1c, s1, s2, dacc, rio);
  }
  if (DOT) {
    __shared__ double sh[3 * 32];
    ed_block_reduce<3>(dacc, sh);
    if (threadIdx.x == 0) {
      partial[blockIdx.x] = dacc[0];
      partial[gridDim.x + blockIdx.x] = dacc[1];
      partial[2 * gridDim.x + blockIdx.x] = dacc[2];
    }
  }
}

// Per-bond operators take the run-time compiled form only (their
// coefficients are immediates of the generated code).
bool ed_lin_supported(const ed_ham* h) {
  return h->mode != ED_HAM_CSR && h->hv_kernel == 2 && h->basis->nspins >= 2 &&
         (!h->bs.per_bond || ed_jit_available());
}

// Launch variants (same results: the integer sums are exact, so the unroll
// depth and register budget change only the speed).
typedef void (*LinKernel)(const uint32_t*, const double*, const double2*, const longlong2*, const int*, int, double2*,
                          int64_t, const uint16_t*, const uint32_t*, const LinSegs, double, double, double*, int);
struct LinVariant {
  LinKernel plain, dot;
  const char* name;
};
static const LinVariant kLinVariants[] = {
    {k_hv_lin<false, 4, 6>, k_hv_lin<true, 4, 5>, "u4-b6"},
    {k_hv_lin<false, 4, 4>, k_hv_lin<true, 4, 4>, "u4-b4"},
    {k_hv_lin<false, 8, 4>, k_hv_lin<true, 8, 4>, "u8-b4"},
    {k_hv_lin<false, 8, 1>, k_hv_lin<true, 8, 1>, "u8-b1"},
};
static const int kNumLinVariants = (int)(sizeof(kLinVariants) / sizeof(kLinVariants[0]));

// Variants kNumLinVariants + 0 .. 4 are the run-time specialised kernel
// (ed_hv_jit.cu) with its five register budgets and block shapes.
static const int kJitVariant = kNumLinVariants;
static const int kNumAllVariants = kNumLinVariants + 5;
static const char* const kJitNames[5] = {"jit", "jit-b4", "jit-b3", "jit-w3", "jit-w4"};
static uint64_t lin_signature(const ed_ham* h);

static int lin_launch(ed_ham* h, int v, const void* x, void* y, bool dot, int sbits, int* nblk_out, bool rio) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  const ed_lin* L = h->lin;
  if (L->per_bond && v < kJitVariant) v = kJitVariant + 1;  // no static per-bond form
  if (v >= kJitVariant)
    return ed_jit_launch(h, lin_signature(h), v - kJitVariant, x, y, dot, sbits, nblk_out, L->segs.word, L->segs.seg,
                         L->segs.w0, rio, L->per_bond ? L->coef.data() : nullptr, L->d_coef, L->pbexp);
  const size_t smem = sizeof(uint16_t) * ((size_t)1 << b->lin_w0);
  LinKernel k = dot ? kLinVariants[v].dot : kLinVariants[v].plain;
  int per_sm = 0;
  ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem));
  if (per_sm < 1) per_sm = 1;
  int64_t g = (b->dim + 255) / 256;
  g = std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx->num_sms * per_sm));
  const int nblk = (int)g;
  if (dot) ED_TRY(ed_ensure_reduce(ctx, (size_t)3 * nblk + 8));
  k<<<nblk, 256, smem, ctx->stream>>>(b->d_states, h->d_diag, (const double2*)x, h->d_xq, h->d_gmax, sbits,
                                      (double2*)y, b->dim, b->d_lin_t0, b->d_lin_t1, L->segs, h->bs.chalf[0],
                                      h->bs.chalf[1], dot ? ctx->d_red : nullptr, rio ? 1 : 0);
  ED_CHECK_LAUNCH(ctx);
  if (nblk_out) *nblk_out = nblk;
  return ED_OK;
}

// Autotuner choices, shared by every operator of the same structure (device,
// sector, bond words): a second Hamiltonian of a lattice does not time again.
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, uint64_t, int, int>, int> g_tune;

static uint64_t lin_signature(const ed_ham* h) {
  uint64_t z = 1469598103934665603ull;  // FNV-1a over the segment table and words
  const LinSegs& sg = h->lin->segs;
  auto mix = [&](uint64_t v) {
    for (int k = 0; k < 8; ++k) { z ^= (v >> (8 * k)) & 0xFF; z *= 1099511628211ull; }
  };
  mix((uint64_t)sg.w0);
  for (int i = 0; i < 7; ++i) mix((uint64_t)sg.seg[i]);
  for (int i = 0; i < sg.seg[6]; ++i) mix(sg.word[i]);
  if (h->lin->per_bond) mix(0x5045524230ull);  // the per-bond form (its couplings are launch parameters)
  return z;
}

// First H.v (and first fused H.v + dot) of a large operator: time each
// variant (two launches after one warm-up, CUDA events on the context's
// stream) and keep the fastest.  The timing synchronises the stream once.
static int lin_autotune(ed_ham* h, const void* x, void* y, int sbits, bool dot, bool rio) {
  ed_lin* L = h->lin;
  ed_ctx* ctx = h->ctx;
  int& chosen = L->variant[2 * (dot ? 1 : 0) + (rio ? 1 : 0)];
  chosen = L->per_bond ? kJitVariant + 1 : 0;
  if (h->basis->dim < (int64_t)1 << 20) return ED_OK;
  const auto key =
      std::make_tuple(ctx->device, h->basis->nspins, h->basis->nup, lin_signature(h), dot ? 1 : 0, rio ? 1 : 0);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      chosen = it->second;
      return ED_OK;
    }
  }
  cudaEvent_t e0, e1;
  ED_CUDA(cudaEventCreate(&e0));
  ED_CUDA(cudaEventCreate(&e1));
  float best = 0.0f;
  int rc = ED_OK;
  bool first = true;
  for (int v = L->per_bond ? kJitVariant : 0; v < kNumAllVariants && rc == ED_OK; ++v) {
    rc = lin_launch(h, v, x, y, dot, sbits, nullptr, rio);
    if (v >= kJitVariant && rc == ED_ENOTSUP) {  // no run-time compiler here: keep the static choice
      rc = ED_OK;
      break;
    }
    if (rc == ED_OK && cudaEventRecord(e0, ctx->stream) != cudaSuccess) rc = ed_fail(ED_ECUDA, "event record");
    for (int it = 0; it < 2 && rc == ED_OK; ++it) rc = lin_launch(h, v, x, y, dot, sbits, nullptr, rio);
    if (rc == ED_OK && cudaEventRecord(e1, ctx->stream) != cudaSuccess) rc = ed_fail(ED_ECUDA, "event record");
    float ms = 0.0f;
    if (rc == ED_OK && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
      rc = ed_fail(ED_ECUDA, "event timing");
    if (rc == ED_OK && (first || ms < best)) {
      best = ms;
      chosen = v;
      first = false;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == ED_OK) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = chosen;
  }
  return rc;
}

// y = H x through the two-table kernel.  With dot set, the kernel also leaves
// per-block partials of Re/Im x^H y and ||y||^2 in ctx->d_red (3 items of
// *nblk_out blocks each, for ed_finish_reduce).
int ed_launch_hv_lin(ed_ham* h, const void* x, void* y, bool dot, int* nblk_out, bool rio) {
  ED_TRY(lin_prepare(h));
  int sbits = 0;
  if (rio && h->xq_src == x) {
    // the fixed-point copy of x was made with it (ed_scale_quantize_r): use it once
    sbits = ed_fx64_sbits(h);
    h->xq_src = nullptr;
  } else if (rio) {
    ED_TRY(ed_fx64_quantize_r(h, (const double*)x, &sbits));
  } else {
    ED_TRY(ed_fx64_quantize(h, (const double2*)x, &sbits));
  }
  const int which = 2 * (dot ? 1 : 0) + (rio ? 1 : 0);
  if (h->lin->variant[which] < 0) ED_TRY(lin_autotune(h, x, y, sbits, dot, rio));
  return lin_launch(h, h->lin->variant[which], x, y, dot, sbits, nblk_out, rio);
}

// Force a launch variant by name ("auto" re-enables the autotuner); for tests
// and tuning.  Returns ED_EINVAL for an unknown name.
int ed_lin_set_variant(ed_ham* h, const char* name) {
  ED_TRY(lin_prepare(h));
  int v = -2;
  if (strcmp(name, "auto") == 0) v = -1;
  for (int i = 0; i < kNumAllVariants - kJitVariant; ++i)
    if (strcmp(name, kJitNames[i]) == 0) v = kJitVariant + i;
  for (int i = 0; i < kNumLinVariants; ++i)
    if (strcmp(name, kLinVariants[i].name) == 0) v = i;
  if (v == -2) return ed_fail(ED_EINVAL, std::string("unknown H.v variant ") + name);
  if (h->lin->per_bond && v >= 0 && v < kJitVariant)
    return ed_fail(ED_ENOTSUP, "per-bond operators have only the run-time compiled H.v variants");
  for (int& c : h->lin->variant) c = v;
  return ED_OK;
}

// The variant last chosen for (dot, real storage); where only one of the two
// storage forms ran, that one.
const char* ed_lin_variant_name(const ed_ham* h, int dot) {
  if (!h->lin) return "";
  const int base = 2 * (dot ? 1 : 0);
  int v = h->lin->variant[base + 1];
  if (v < 0) v = h->lin->variant[base];
  if (v < 0) return "";
  if (v >= kJitVariant) return kJitNames[v - kJitVariant];
  return kLinVariants[v].name;
}

void ed_lin_invalidate(ed_lin* L) {
  if (L) L->built_nb = -1;
}
