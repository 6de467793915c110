// Hamiltonian application on the device.
//
//   H = sum_{(i,j) in nn}  [ J1/2 (S+_i S-_j + h.c.) + D1 S^z_i S^z_j ]
//     + sum_{(i,j) in nnn} [ J2/2 (S+_i S-_j + h.c.) + D2 S^z_i S^z_j ]
//     + sum_i h_i S^z_i
//
// Matrix elements follow the reference exactly:
//  * diagonal: build_diag (include/hamiltonian.tmpl_func.hpp:129-225) and
//    build_disorder (ibid :97-125, src/hamiltonian.cpp:31-49); computed with
//    explicitly rounded FP64 operations so no multiply-add is contracted,
//    reproducing the reference's separately rounded products and sums;
//  * off-diagonal: J*0.5 for every antiparallel bond, the column being the
//    rank of the state with both bits flipped (get_coup_elems,
//    ibid :350-387, src/hamiltonian.cpp:72-99); duplicated bonds add up in
//    the reference's nn-pass-then-nnn-pass ADD_VALUES order (ibid :229-344).
#include "ed_internal.h"
#include "ed_device.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

struct DiagParams {
  int nb;
  int N;
  int mode;                  // 0 zero, 1 build_diag, 2 build_disorder, 3 per-bond
  int has_hi;
  uint32_t mask[ED_MAX_BONDS];
  uint8_t type[ED_MAX_BONDS];  // 0 nn, 1 nnn
  double D1, D2;
  double Db[ED_MAX_BONDS];
  double hi[ED_MAX_SPINS];
};

// ---------------------------------------------------------------------------
// Diagonal
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ed_disorder_elem(uint32_t s, const DiagParams& p) {
  // src/hamiltonian.cpp:38-46: sequential +h_i / -h_i
  double d = 0.0;
  for (int i = 0; i < p.N; ++i) d = ((s >> i) & 1u) ? __dadd_rn(d, p.hi[i]) : __dsub_rn(d, p.hi[i]);
  return d;
}

__device__ __forceinline__ double ed_diag_value(uint32_t s, const DiagParams& p, bool* has_entry) {
  if (p.mode == 3) {
    double d = 0.0;
    for (int b = 0; b < p.nb; ++b) {
      uint32_t t = s & p.mask[b];
      double sg = (t != 0u && t != p.mask[b]) ? -1.0 : 1.0;
      d = __dadd_rn(d, __dmul_rn(__dmul_rn(p.Db[b], 0.25), sg));
    }
    if (p.has_hi) d = __dadd_rn(d, __dmul_rn(0.5, ed_disorder_elem(s, p)));
    *has_entry = true;
    return d;
  }
  int n1 = 0, a1 = 0, n2 = 0, a2 = 0;
  for (int b = 0; b < p.nb; ++b) {
    uint32_t t = s & p.mask[b];
    int anti = (t != 0u && t != p.mask[b]) ? 1 : 0;
    if (p.type[b] == 0) { ++n1; a1 += anti; } else { ++n2; a2 += anti; }
  }
  const double e1 = (double)(n1 - 2 * a1), e2 = (double)(n2 - 2 * a2);
  if (p.mode == 2) {
    // Delta1*0.25*tmp1 + Delta2*0.25*tmp2 + 0.5*disorder (tmpl_func.hpp:111)
    double a = __dmul_rn(__dmul_rn(p.D1, 0.25), e1);
    double b = __dmul_rn(__dmul_rn(p.D2, 0.25), e2);
    double c = __dmul_rn(0.5, ed_disorder_elem(s, p));
    *has_entry = true;
    return __dadd_rn(__dadd_rn(a, b), c);
  }
  if (p.mode == 1) {
    double d = 0.0;
    bool any = false;
    if (!(fabs(p.D1) < 1e-14 && fabs(p.D2) < 1e-14)) {
      if (fabs(p.D1) >= 1e-14 && e1 != 0.0) { d = __dadd_rn(d, __dmul_rn(__dmul_rn(p.D1, 0.25), e1)); any = true; }
      if (fabs(p.D2) >= 1e-14 && e2 != 0.0) { d = __dadd_rn(d, __dmul_rn(__dmul_rn(p.D2, 0.25), e2)); any = true; }
    }
    *has_entry = any;
    return d;
  }
  *has_entry = false;
  return 0.0;
}

__global__ void k_build_diag(const uint32_t* __restrict__ states, int64_t dim, const DiagParams p,
                             double* __restrict__ diag) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    bool he;
    diag[r] = ed_diag_value(states[r], p, &he);
  }
}

static void make_diag_params(const ed_ham* h, DiagParams& p) {
  memset(&p, 0, sizeof(p));
  p.N = h->basis->nspins;
  p.nb = (int)h->bi.size();
  for (int b = 0; b < p.nb; ++b) {
    p.mask[b] = (1u << h->bi[b]) | (1u << h->bj[b]);
    p.type[b] = h->per_bond ? 0 : (uint8_t)h->btype[b];
    if (h->per_bond) p.Db[b] = h->bD[b];
  }
  p.D1 = h->D1;
  p.D2 = h->D2;
  p.has_hi = h->disorder ? 1 : 0;
  for (int i = 0; i < p.N && h->disorder; ++i) p.hi[i] = h->hi[i];
  if (h->per_bond) p.mode = 3;
  else if (h->disorder) p.mode = 2;
  else if (h->diag_built) p.mode = 1;
  else p.mode = 0;
}

static int grid_cap(ed_ctx* ctx, int64_t n, int threads, int per_sm) {
  int64_t g = (n + threads - 1) / threads;
  int64_t cap = (int64_t)ctx->num_sms * per_sm;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

int ed_launch_build_diag(ed_ham* h) {
  ed_ctx* ctx = h->ctx;
  DiagParams p;
  make_diag_params(h, p);
  k_build_diag<<<grid_cap(ctx, h->basis->dim, 256, 8), 256, 0, ctx->stream>>>(h->basis->d_states, h->basis->dim, p,
                                                                              h->d_diag);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Off-diagonal bond set for H.v.
// ---------------------------------------------------------------------------
static void bond_chunks(const RankTables& rt, BondSet& bs, int b, int i, int j) {
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  int ci = 0, cj = 0;
  for (int k = 0; k < rt.K; ++k) {
    if (lo >= rt.off[k] && lo < rt.off[k] + rt.w[k]) ci = k;
    if (hi >= rt.off[k] && hi < rt.off[k] + rt.w[k]) cj = k;
  }
  bs.ci[b] = (uint8_t)ci;
  bs.cj[b] = (uint8_t)cj;
  bs.lo[b] = (uint8_t)lo;
  const uint32_t m = (1u << i) | (1u << j);
  for (int k = 0; k < ED_RANK_MAX_CHUNKS; ++k)
    bs.xm[b][k] = k < rt.K ? (uint16_t)((m >> rt.off[k]) & ((1u << rt.w[k]) - 1u)) : 0;
}

void ed_ham_make_bondset(ed_ham* h) {
  BondSet& bs = h->bs;
  memset(&bs, 0, sizeof(bs));
  ed_lin_invalidate(h->lin);
  if (!h->offdiag_built) return;
  const RankTables& rt = h->basis->rt;
  if (h->per_bond) {
    bs.per_bond = 1;
    for (size_t b = 0; b < h->bi.size(); ++b) {
      bs.mask[bs.nb] = (1u << h->bi[b]) | (1u << h->bj[b]);
      bs.type[bs.nb] = (uint8_t)bs.nb;
      bs.chalf[bs.nb] = h->bJ[b] * 0.5;
      bond_chunks(rt, bs, bs.nb, h->bi[b], h->bj[b]);
      ++bs.nb;
    }
    bs.ntypes = bs.nb;
    return;
  }
  bs.ntypes = 2;
  bs.chalf[0] = h->J1 * 0.5;
  bs.chalf[1] = h->J2 * 0.5;
  for (size_t b = 0; b < h->bi.size(); ++b) {
    int t = h->btype[b];
    double J = t == 0 ? h->J1 : h->J2;
    if (std::fabs(J) < 1e-14) continue;  // pass skipped (tmpl_func.hpp:246, 280)
    bs.mask[bs.nb] = (1u << h->bi[b]) | (1u << h->bj[b]);
    bs.type[bs.nb] = (uint8_t)t;
    bond_chunks(rt, bs, bs.nb, h->bi[b], h->bj[b]);
    ++bs.nb;
  }
  // segments for the fixed-point kernel (order within a row is irrelevant
  // there: integer sums are exact)
  BondSegments& sg = h->segs;
  memset(&sg, 0, sizeof(sg));
  int n = 0, cls = 0;
  for (int ci = 0; ci < ED_RANK_MAX_CHUNKS; ++ci)
    for (int cj = ci; cj < ED_RANK_MAX_CHUNKS; ++cj, ++cls)
      for (int t = 0; t < 2; ++t) {
        sg.seg[cls * 2 + t] = n;
        for (int b = 0; b < bs.nb; ++b) {
          if (bs.ci[b] != ci || bs.cj[b] != cj || bs.type[b] != t) continue;
          if (__builtin_popcount(bs.mask[b]) != 2) continue;  // i == j never couples
          sg.word[n++] = (unsigned long long)bs.mask[b] | ((unsigned long long)bs.xm[b][ci] << 32) |
                         ((unsigned long long)bs.xm[b][cj] << 48);
        }
      }
  sg.seg[2 * ED_NCLASS] = n;
}

void ed_ham_unique_masks(const ed_ham* h, std::vector<uint32_t>& masks, std::vector<double>& vals) {
  masks.clear();
  vals.clear();
  const BondSet& bs = h->bs;
  for (int b = 0; b < bs.nb; ++b) {
    uint32_t m = bs.mask[b];
    double v = bs.chalf[bs.type[b]];
    if (__builtin_popcount(m) != 2) continue;  // i == j never couples
    size_t k = 0;
    for (; k < masks.size(); ++k)
      if (masks[k] == m) break;
    if (k == masks.size()) { masks.push_back(m); vals.push_back(0.0 + v); }
    else vals[k] = vals[k] + v;
  }
}

// ---------------------------------------------------------------------------
// Matrix-free H.v: one thread per basis state; rank tables in shared memory;
// gathers x at the ranks of the bond-flipped states.
// ---------------------------------------------------------------------------
template <int K, bool PERBOND>
__global__ void __launch_bounds__(256) k_hv_gather(const uint32_t* __restrict__ states, const double* __restrict__ diag,
                                                   const double2* __restrict__ x, double2* __restrict__ y,
                                                   int64_t dim, const RankTables rt, const BondSet bs) {
  extern __shared__ uint32_t stab[];
  ed_load_tables(stab, rt);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const uint32_t s = states[r];
    RowRank<K> R;
    ed_row_rank<K>(s, stab, rt, R);
    double a0r = 0.0, a0i = 0.0, a1r = 0.0, a1i = 0.0;
#pragma unroll 4
    for (int b = 0; b < bs.nb; ++b) {
      const uint32_t m = bs.mask[b];
      const uint32_t t = s & m;
      if (t != 0u && t != m) {
        const uint32_t c = ed_rank_flip<K>((uint32_t)r, s, stab, rt, R, bs, b);
        const double2 v = __ldg(&x[c]);
        if (PERBOND) {
          const double ch = bs.chalf[b];
          a0r = fma(ch, v.x, a0r);
          a0i = fma(ch, v.y, a0i);
        } else if (bs.type[b] == 0) {
          a0r += v.x; a0i += v.y;
        } else {
          a1r += v.x; a1i += v.y;
        }
      }
    }
    const double d = diag[r];
    const double2 xv = x[r];
    double yr, yi;
    if (PERBOND) {
      yr = fma(d, xv.x, a0r);
      yi = fma(d, xv.y, a0i);
    } else {
      yr = fma(d, xv.x, fma(bs.chalf[0], a0r, bs.chalf[1] * a1r));
      yi = fma(d, xv.y, fma(bs.chalf[0], a0i, bs.chalf[1] * a1i));
    }
    y[r] = make_double2(yr, yi);
  }
}

template <int K, bool PB>
static int launch_hv_k(ed_ham* h, const double2* x, double2* y) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  size_t smem = (size_t)b->rt.total * sizeof(uint32_t);
  static bool attr_set[2][5] = {{false}};
  if (!attr_set[PB][K]) {
    ED_CUDA(cudaFuncSetAttribute(k_hv_gather<K, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(56 * 1024)));
    attr_set[PB][K] = true;
  }
  int per_sm = 0;
  ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_gather<K, PB>, 256, smem));
  if (per_sm < 1) per_sm = 1;
  int grid = grid_cap(ctx, b->dim, 256, per_sm);
  k_hv_gather<K, PB><<<grid, 256, smem, ctx->stream>>>(b->d_states, h->d_diag, x, y, b->dim, b->rt, h->bs);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Exact integer accumulation.  FP64 adds run at 1/64 of the integer rate on
// this part, and a row sums ~60 gathered complex entries, so the sums are
// formed exactly in 128-bit integers instead:
//  1. k_quantize stores x as block floating point: for each 32-state block,
//     Eb = largest biased exponent of the 64 doubles, and each double v is
//     kept as q = v * 2^(61 - (Eb - 1023)), a 62-bit two's complement integer
//     (|q| < 2^62), truncating bits below 2^(Eb - 1084) (relative to the
//     block's largest entry: 2^-61).
//  2. k_hv_fixed gathers q and its block exponent, aligns it to a common
//     scale 2^(G - 1084 - 40) (G = largest block exponent of the vector) and
//     adds it into a 128-bit accumulator per coupling type — exactly.
//  3. Each sum is rounded once to FP64, scaled, and combined with the
//     diagonal term in FP64.
// Zero and subnormal entries quantize to 0.  A non-finite entry is stored as
// the sentinel INT64_MIN (outside the mantissa range) and does not enter the
// block exponent; any row that gathers it returns NaN.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_quantize(const double2* __restrict__ x, int64_t dim, longlong2* __restrict__ xq,
                                                  uint16_t* __restrict__ xe, int* __restrict__ gmax) {
  const int lane = threadIdx.x & 31;
  const int64_t nblk = (dim + 31) >> 5;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int wmax = 0;
  for (int64_t bk = warp; bk < nblk; bk += nwarps) {
    const int64_t r = (bk << 5) + lane;
    const bool valid = r < dim;
    const double2 v = valid ? x[r] : make_double2(0.0, 0.0);
    const unsigned long long br = (unsigned long long)__double_as_longlong(v.x);
    const unsigned long long bi = (unsigned long long)__double_as_longlong(v.y);
    const int er = (int)((br >> 52) & 0x7FF), ei = (int)((bi >> 52) & 0x7FF);
    const int fr = er == 0x7FF ? 0 : er, fi = ei == 0x7FF ? 0 : ei;  // finite exponents only
    const int eb = (int)__reduce_max_sync(0xffffffffu, (unsigned)max(fr, fi));
    long long q[2];
    const unsigned long long bits[2] = {br, bi};
    const int ex[2] = {er, ei};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      long long m = 0;
      if (ex[k] == 0x7FF) {
        m = (long long)0x8000000000000000ull;
      } else if (ex[k] != 0) {
        const unsigned long long mant = (bits[k] & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
        const int sh = ex[k] - eb + 9;  // q = mant * 2^sh, sh <= 9
        unsigned long long a = sh >= 0 ? (mant << sh) : (sh > -64 ? (mant >> (-sh)) : 0ull);
        m = (long long)a;
        if (bits[k] >> 63) m = -m;
      }
      q[k] = m;
    }
    if (valid) xq[r] = make_longlong2(q[0], q[1]);
    if (lane == 0) xe[bk] = (uint16_t)eb;
    wmax = max(wmax, eb);
  }
  // one atomic per warp
  if (lane == 0 && wmax > 0) atomicMax(gmax, wmax);
}

struct Acc128 {
  unsigned long long lo;
  long long hi;
};

__device__ __forceinline__ void acc_add(Acc128& a, long long q, int shift) {
  // a += q * 2^shift (shift in [-63, 40]), exact for shift >= 0
  unsigned long long lo;
  long long hi;
  if (shift >= 0) {
    lo = (unsigned long long)q << shift;
    hi = shift == 0 ? (q >> 63) : (q >> (64 - shift));
  } else {
    const long long t = shift > -63 ? (q >> (-shift)) : (q >> 63);
    lo = (unsigned long long)t;
    hi = t >> 63;
  }
  const unsigned long long nlo = a.lo + lo;
  a.hi = a.hi + hi + (nlo < lo ? 1 : 0);
  a.lo = nlo;
}

__device__ __forceinline__ double acc_to_double(const Acc128& a) {
  // hi * 2^64 is exact (|hi| < 2^53); one rounding for the low word, one for the sum
  return fma((double)a.hi, 18446744073709551616.0, (double)a.lo);
}

template <int K>
__global__ void __launch_bounds__(256) k_hv_fixed(const uint32_t* __restrict__ states, const double* __restrict__ diag,
                                                  const double2* __restrict__ x, const longlong2* __restrict__ xq,
                                                  const uint16_t* __restrict__ xe, const int* __restrict__ gmax_p,
                                                  double2* __restrict__ y, int64_t dim, const RankTables rt,
                                                  const BondSet bs) {
  extern __shared__ uint32_t stab[];
  ed_load_tables(stab, rt);
  const int gmax = *gmax_p;
  // value of one accumulator unit: 2^(gmax - 1084 - 40), split to stay normal
  const int e_unit = gmax - 1124;
  const double s1 = __longlong_as_double((long long)(e_unit / 2 + 1023) << 52);
  const double s2 = __longlong_as_double((long long)(e_unit - e_unit / 2 + 1023) << 52);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const uint32_t s = states[r];
    RowRank<K> R;
    ed_row_rank<K>(s, stab, rt, R);
    Acc128 a0r = {0, 0}, a0i = {0, 0}, a1r = {0, 0}, a1i = {0, 0};
    bool bad = false;
#pragma unroll 4
    for (int b = 0; b < bs.nb; ++b) {
      const uint32_t m = bs.mask[b];
      const uint32_t t = s & m;
      if (t != 0u && t != m) {
        const uint32_t c = ed_rank_flip<K>((uint32_t)r, s, stab, rt, R, bs, b);
        const longlong2 q = __ldg(&xq[c]);
        const int eb = (int)__ldg(&xe[c >> 5]);
        bad |= (q.x == (long long)0x8000000000000000ull) | (q.y == (long long)0x8000000000000000ull);
        const int sh = eb - gmax + 40;
        if (bs.type[b] == 0) {
          acc_add(a0r, q.x, sh);
          acc_add(a0i, q.y, sh);
        } else {
          acc_add(a1r, q.x, sh);
          acc_add(a1i, q.y, sh);
        }
      }
    }
    const double d = diag[r];
    const double2 xv = x[r];
    const double s0r = acc_to_double(a0r) * s1 * s2, s0i = acc_to_double(a0i) * s1 * s2;
    const double s1r = acc_to_double(a1r) * s1 * s2, s1i = acc_to_double(a1i) * s1 * s2;
    double yr = fma(d, xv.x, fma(bs.chalf[0], s0r, bs.chalf[1] * s1r));
    double yi = fma(d, xv.y, fma(bs.chalf[0], s0i, bs.chalf[1] * s1i));
    if (bad) { yr = __longlong_as_double(0x7FF8000000000000ll); yi = yr; }
    y[r] = make_double2(yr, yi);
  }
}

// ---------------------------------------------------------------------------
// 64-bit fixed point: x is quantised once per H.v against its largest entry,
// q = round(v * 2^(S - (Emax - 1022))) with |q| <= 2^S, where 2^(Emax-1022)
// bounds every |v| and S = 62 - ceil(log2(max bonds per coupling type + 1)),
// so a row's sum of one coupling type cannot overflow int64.  Each gathered
// term is then one 64-bit add; the sums are exact and rounded once to FP64.
// Quantisation error per entry <= 2^-(S+1) of the largest |v|.
// ---------------------------------------------------------------------------
// gmax[0] = largest finite biased exponent, gmax[1] |= some entry not
// finite, and with imag != nullptr *imag |= some imaginary part nonzero.
__global__ void __launch_bounds__(256) k_max_exponent(const double2* __restrict__ x, int64_t dim,
                                                      int* __restrict__ gmax, int* __restrict__ nonfinite,
                                                      int* __restrict__ imag) {
  int m = 0, nf = 0, im = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const double2 v = x[r];
    const int er = (int)(((unsigned long long)__double_as_longlong(v.x) >> 52) & 0x7FF);
    const int ei = (int)(((unsigned long long)__double_as_longlong(v.y) >> 52) & 0x7FF);
    nf |= (er == 0x7FF) | (ei == 0x7FF);
    im |= v.y != 0.0;
    m = max(m, max(er == 0x7FF ? 0 : er, ei == 0x7FF ? 0 : ei));
  }
  m = (int)__reduce_max_sync(0xffffffffu, (unsigned)m);
  nf = (int)__reduce_or_sync(0xffffffffu, (unsigned)nf);
  im = (int)__reduce_or_sync(0xffffffffu, (unsigned)im);
  if ((threadIdx.x & 31) == 0) {
    if (m > 0) atomicMax(gmax, m);
    if (nf) atomicOr(nonfinite, 1);
    if (im && imag) atomicOr(imag, 1);
  }
}

// With imag_p != nullptr and *imag_p == 0 (every imaginary part zero) only
// the real parts are stored, as int64[dim] at the start of xq.
__global__ void __launch_bounds__(256) k_quantize64(const double2* __restrict__ x, int64_t dim, const int* __restrict__ gmax_p,
                                                    int sbits, longlong2* __restrict__ xq, const int* __restrict__ imag_p) {
  const int emax = *gmax_p;
  const bool real_only = imag_p && *imag_p == 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const double2 v = x[r];
    const unsigned long long bits[2] = {(unsigned long long)__double_as_longlong(v.x),
                                        (unsigned long long)__double_as_longlong(v.y)};
    long long q[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int e = (int)((bits[k] >> 52) & 0x7FF);
      long long m = 0;
      if (e == 0x7FF) {
        m = (long long)0x8000000000000000ull;  // non-finite sentinel
      } else if (e != 0) {
        const unsigned long long mant = (bits[k] & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
        const int sh = e - emax + sbits - 53;  // q = mant * 2^sh, sh <= sbits - 53
        unsigned long long a;
        if (sh >= 0) a = mant << sh;
        else if (sh > -63) a = (mant + (1ull << (-sh - 1))) >> (-sh);  // round half up in magnitude
        else a = 0;
        m = (long long)a;
        if (bits[k] >> 63) m = -m;
      }
      q[k] = m;
    }
    if (real_only) ((long long*)xq)[r] = q[0];
    else xq[r] = make_longlong2(q[0], q[1]);
  }
}

// One (chunk class, type) segment of the fixed-point kernel: rank of the
// flipped state from the row's rank (only chunks CI..CJ change), predicated
// gathers four bonds at a time so several loads are in flight per thread.
template <int K, int CI, int CJ>
__device__ __forceinline__ void fx64_segment(const BondSegments& sg, int b0, int b1, uint32_t s, uint32_t r,
                                             const uint32_t* __restrict__ stab, const RankTables& rt,
                                             const RowRank<K>& R, const longlong2* __restrict__ xq, long long& ar,
                                             long long& ai, bool& bad) {
  constexpr int U = 4;
  const long long kNaN = (long long)0x8000000000000000ull;
  for (int b = b0; b < b1; b += U) {
    uint32_t c[U];
    bool on[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const bool inb = b + u < b1;
      const unsigned long long w = inb ? sg.word[b + u] : 0ull;
      const uint32_t m = (uint32_t)w;
      const uint32_t t = s & m;
      on[u] = inb && t != 0u && t != m;
      uint32_t rr = r;
      if (CI == CJ) {
        const uint32_t cc = R.cv[CI] ^ (uint32_t)((w >> 32) & 0xFFFFu);
        rr += stab[ed_tab_index<K>(rt, CI, R.pc[CI], cc)] - R.tv[CI];
      } else {
        const int d = (s & m & (0u - m)) ? -1 : 1;  // lowest bond bit set -> one fewer below
#pragma unroll
        for (int k = CI; k <= CJ; ++k) {
          uint32_t cc = R.cv[k];
          if (k == CI) cc ^= (uint32_t)((w >> 32) & 0xFFFFu);
          if (k == CJ) cc ^= (uint32_t)(w >> 48);
          const int p = R.pc[k] + (k > CI ? d : 0);
          rr += stab[ed_tab_index<K>(rt, k, p, cc)] - R.tv[k];
        }
      }
      c[u] = on[u] ? rr : r;
    }
    longlong2 q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) q[u] = on[u] ? __ldg(&xq[c[u]]) : make_longlong2(0, 0);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      bad |= (q[u].x == kNaN) | (q[u].y == kNaN);
      ar += q[u].x;
      ai += q[u].y;
    }
  }
}

template <int K, int CI, int CJ>
__device__ __forceinline__ void fx64_class(const BondSegments& sg, uint32_t s, uint32_t r, const uint32_t* stab,
                                           const RankTables& rt, const RowRank<K>& R, const longlong2* xq,
                                           long long (&a)[4], bool& bad) {
  if (CJ >= K) return;
  constexpr int cls = CI * (2 * ED_RANK_MAX_CHUNKS - CI + 1) / 2 + (CJ - CI);
  fx64_segment<K, CI, CJ>(sg, sg.seg[2 * cls], sg.seg[2 * cls + 1], s, r, stab, rt, R, xq, a[0], a[1], bad);
  fx64_segment<K, CI, CJ>(sg, sg.seg[2 * cls + 1], sg.seg[2 * cls + 2], s, r, stab, rt, R, xq, a[2], a[3], bad);
}

template <int K>
__global__ void __launch_bounds__(256) k_hv_fx64(const uint32_t* __restrict__ states, const double* __restrict__ diag,
                                                 const double2* __restrict__ x, const longlong2* __restrict__ xq,
                                                 const int* __restrict__ gmax_p, int sbits, double2* __restrict__ y,
                                                 int64_t dim, const RankTables rt, const BondSegments sg,
                                                 double c0, double c1) {
  extern __shared__ uint32_t stab[];
  ed_load_tables(stab, rt);
  // one unit = 2^(emax - 1022 - sbits), applied as two normal factors
  const int e_unit = *gmax_p - 1022 - sbits;
  const double s1 = __longlong_as_double((long long)(e_unit / 2 + 1023) << 52);
  const double s2 = __longlong_as_double((long long)(e_unit - e_unit / 2 + 1023) << 52);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const uint32_t s = states[r];
    RowRank<K> R;
    ed_row_rank<K>(s, stab, rt, R);
    long long a[4] = {0, 0, 0, 0};  // nn re, nn im, nnn re, nnn im
    bool bad = false;
    const uint32_t rr = (uint32_t)r;
    fx64_class<K, 0, 0>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 1, 1>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 2, 2>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 3, 3>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 0, 1>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 1, 2>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 2, 3>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 0, 2>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 1, 3>(sg, s, rr, stab, rt, R, xq, a, bad);
    fx64_class<K, 0, 3>(sg, s, rr, stab, rt, R, xq, a, bad);
    const double d = diag[r];
    const double2 xv = x[r];
    const double s0r = (double)a[0] * s1 * s2, s0i = (double)a[1] * s1 * s2;
    const double s1r = (double)a[2] * s1 * s2, s1i = (double)a[3] * s1 * s2;
    double yr = fma(d, xv.x, fma(c0, s0r, c1 * s1r));
    double yi = fma(d, xv.y, fma(c0, s0i, c1 * s1i));
    if (bad) { yr = __longlong_as_double(0x7FF8000000000000ll); yi = yr; }
    y[r] = make_double2(yr, yi);
  }
}

static int ensure_fixed_buffers(ed_ham* h) {
  const int64_t dim = h->basis->dim;
  if (!h->d_xq) {
    if (cudaMalloc(&h->d_xq, sizeof(longlong2) * (size_t)dim) != cudaSuccess ||
        cudaMalloc(&h->d_xe, sizeof(uint16_t) * (size_t)((dim + 31) / 32)) != cudaSuccess ||
        cudaMalloc(&h->d_gmax, 4 * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return ed_fail(ED_ENOMEM, "H.v scratch does not fit in device memory");
    }
  }
  return ED_OK;
}

template <int K>
static int launch_hv_fixed_k(ed_ham* h, const double2* x, double2* y) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  ED_TRY(ensure_fixed_buffers(h));
  h->xq_src = nullptr;
  ED_CUDA(cudaMemsetAsync(h->d_gmax, 0, sizeof(int), ctx->stream));
  k_quantize<<<grid_cap(ctx, b->dim, 256, 8), 256, 0, ctx->stream>>>(x, b->dim, h->d_xq, h->d_xe, h->d_gmax);
  ED_CHECK_LAUNCH(ctx);
  size_t smem = (size_t)b->rt.total * sizeof(uint32_t);
  static bool attr_set[5] = {false};
  if (!attr_set[K]) {
    ED_CUDA(cudaFuncSetAttribute(k_hv_fixed<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(56 * 1024)));
    attr_set[K] = true;
  }
  int per_sm = 0;
  ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_fixed<K>, 256, smem));
  if (per_sm < 1) per_sm = 1;
  k_hv_fixed<K><<<grid_cap(ctx, b->dim, 256, per_sm), 256, smem, ctx->stream>>>(
      b->d_states, h->d_diag, x, h->d_xq, h->d_xe, h->d_gmax, y, b->dim, b->rt, h->bs);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

// Largest number of bonds of one coupling type, for the fixed-point headroom.
static int max_type_count(const BondSet& bs) {
  int c[2] = {0, 0};
  for (int b = 0; b < bs.nb; ++b) c[bs.type[b] & 1]++;
  return c[0] > c[1] ? c[0] : c[1];
}

// The same two passes for a real input stored as double[dim] (real-mode
// solves): the imaginary-nonzero flag stays 0, only real parts are written.
__global__ void __launch_bounds__(256) k_max_exponent_r(const double* __restrict__ x, int64_t dim,
                                                        int* __restrict__ gmax, int* __restrict__ nonfinite) {
  int m = 0, nf = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const int e = (int)(((unsigned long long)__double_as_longlong(x[r]) >> 52) & 0x7FF);
    nf |= e == 0x7FF;
    m = max(m, e == 0x7FF ? 0 : e);
  }
  m = (int)__reduce_max_sync(0xffffffffu, (unsigned)m);
  nf = (int)__reduce_or_sync(0xffffffffu, (unsigned)nf);
  if ((threadIdx.x & 31) == 0) {
    if (m > 0) atomicMax(gmax, m);
    if (nf) atomicOr(nonfinite, 1);
  }
}

// One entry in 64-bit fixed point: v * 2^(sbits - 1 - (emax - 1023)) rounded,
// or the non-finite sentinel.
__device__ __forceinline__ long long ed_fx64_entry(double v, int emax, int sbits) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((bits >> 52) & 0x7FF);
  long long m = 0;
  if (e == 0x7FF) {
    m = (long long)0x8000000000000000ull;  // non-finite sentinel
  } else if (e != 0) {
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    const int sh = e - emax + sbits - 53;
    unsigned long long a;
    if (sh >= 0) a = mant << sh;
    else if (sh > -63) a = (mant + (1ull << (-sh - 1))) >> (-sh);  // round half up in magnitude
    else a = 0;
    m = (long long)a;
    if (bits >> 63) m = -m;
  }
  return m;
}

__global__ void __launch_bounds__(256) k_quantize64_r(const double* __restrict__ x, int64_t dim,
                                                      const int* __restrict__ gmax_p, int sbits,
                                                      long long* __restrict__ xq) {
  const int emax = *gmax_p;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride)
    xq[r] = ed_fx64_entry(x[r], emax, sbits);
}

// dst = src * s and its fixed-point copy with the largest exponent emax
// (found on the host); the flags of gmax as k_max_exponent_r leaves them for
// a finite real input.
__global__ void __launch_bounds__(256) k_scale_quantize_r(const double* __restrict__ src, double* __restrict__ dst,
                                                          double s, int64_t dim, int emax, int sbits,
                                                          long long* __restrict__ xq, int* __restrict__ gmax) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    gmax[0] = emax;
    gmax[1] = 0;
    gmax[2] = 0;
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const double v = src[r] * s;
    dst[r] = v;
    xq[r] = ed_fx64_entry(v, emax, sbits);
  }
}

int ed_fx64_sbits(const ed_ham* h) {
  int head = 0;
  while ((1 << head) < max_type_count(h->bs) + 1) ++head;
  return 62 - head;
}

int ed_fx64_emax_scaled(double absmax_hi, double s) {
  uint64_t lb;
  std::memcpy(&lb, &absmax_hi, sizeof(lb));
  const uint64_t ub = lb | 0xFFFFFFFFull;
  double u;
  std::memcpy(&u, &ub, sizeof(u));
  const double ml = absmax_hi * s, mu = u * s;
  if (!std::isfinite(ml) || !std::isfinite(mu) || !(s > 0.0)) return -1;
  uint64_t bl, bu;
  std::memcpy(&bl, &ml, sizeof(bl));
  std::memcpy(&bu, &mu, sizeof(bu));
  const int el = (int)((bl >> 52) & 0x7FF), eu = (int)((bu >> 52) & 0x7FF);
  return el == eu ? el : -1;
}

int ed_scale_quantize_r(ed_ham* h, const double* src, double* dst, double s, double src_absmax_hi) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  const int emax = ed_fx64_emax_scaled(src_absmax_hi, s);
  if (emax < 0) return ED_ENOTSUP;  // not determined: the caller scales and the H.v quantizes
  ED_TRY(ensure_fixed_buffers(h));
  const int g = grid_cap(ctx, b->dim, 256, 8);
  k_scale_quantize_r<<<g, 256, 0, ctx->stream>>>(src, dst, s, b->dim, emax, ed_fx64_sbits(h), (long long*)h->d_xq,
                                                  h->d_gmax);
  ED_CHECK_LAUNCH(ctx);
  h->xq_src = dst;
  return ED_OK;
}

int ed_fx64_quantize_r(ed_ham* h, const double* x, int* sbits) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  ED_TRY(ensure_fixed_buffers(h));
  h->xq_src = nullptr;
  *sbits = ed_fx64_sbits(h);
  ED_CUDA(cudaMemsetAsync(h->d_gmax, 0, 3 * sizeof(int), ctx->stream));
  const int g = grid_cap(ctx, b->dim, 256, 8);
  k_max_exponent_r<<<g, 256, 0, ctx->stream>>>(x, b->dim, h->d_gmax, h->d_gmax + 1);
  ED_CHECK_LAUNCH(ctx);
  k_quantize64_r<<<g, 256, 0, ctx->stream>>>(x, b->dim, h->d_gmax, *sbits, (long long*)h->d_xq);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

int ed_fx64_quantize(ed_ham* h, const double2* x, int* sbits) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  ED_TRY(ensure_fixed_buffers(h));
  h->xq_src = nullptr;
  *sbits = ed_fx64_sbits(h);
  ED_CUDA(cudaMemsetAsync(h->d_gmax, 0, 3 * sizeof(int), ctx->stream));
  const int g = grid_cap(ctx, b->dim, 256, 8);
  k_max_exponent<<<g, 256, 0, ctx->stream>>>(x, b->dim, h->d_gmax, h->d_gmax + 1, h->d_gmax + 2);
  ED_CHECK_LAUNCH(ctx);
  k_quantize64<<<g, 256, 0, ctx->stream>>>(x, b->dim, h->d_gmax, *sbits, h->d_xq, h->d_gmax + 2);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

static int launch_hv_dispatch(ed_ham* h, const double2* x, double2* y) {
  if (h->mode == ED_HAM_CSR && h->d_rowptr) return ed_launch_csr_spmv(h, x, y);
  const bool pb = h->bs.per_bond != 0;
  if (ed_lin_supported(h)) return ed_launch_hv_lin(h, x, y, false, nullptr, false);
  if (!pb && h->hv_kernel == 1) {
    switch (h->basis->rt.K) {
      case 1: return launch_hv_fixed_k<1>(h, x, y);
      case 2: return launch_hv_fixed_k<2>(h, x, y);
      case 3: return launch_hv_fixed_k<3>(h, x, y);
      default: return launch_hv_fixed_k<4>(h, x, y);
    }
  }
  switch (h->basis->rt.K) {
    case 1: return pb ? launch_hv_k<1, true>(h, x, y) : launch_hv_k<1, false>(h, x, y);
    case 2: return pb ? launch_hv_k<2, true>(h, x, y) : launch_hv_k<2, false>(h, x, y);
    case 3: return pb ? launch_hv_k<3, true>(h, x, y) : launch_hv_k<3, false>(h, x, y);
    default: return pb ? launch_hv_k<4, true>(h, x, y) : launch_hv_k<4, false>(h, x, y);
  }
}

int ed_launch_hv_r(ed_ham* h, const double* x, double* y) {
  if (!ed_lin_supported(h)) return ed_fail(ED_ENOTSUP, "real-storage H.v needs the two-table fixed-point kernel");
  ed_ctx* ctx = h->ctx;
  if (!ctx->profiling) return ed_launch_hv_lin(h, x, y, false, nullptr, true);
  cudaEvent_t e0, e1;
  ED_CUDA(cudaEventCreate(&e0));
  ED_CUDA(cudaEventCreate(&e1));
  ED_CUDA(cudaEventRecord(e0, ctx->stream));
  int rc = ed_launch_hv_lin(h, x, y, false, nullptr, true);
  ED_CUDA(cudaEventRecord(e1, ctx->stream));
  ctx->prof_events.push_back(e0);
  ctx->prof_events.push_back(e1);
  return rc;
}

int ed_launch_hv(ed_ham* h, const double2* x, double2* y) {
  ed_ctx* ctx = h->ctx;
  if (!ctx->profiling) return launch_hv_dispatch(h, x, y);
  cudaEvent_t e0, e1;
  ED_CUDA(cudaEventCreate(&e0));
  ED_CUDA(cudaEventCreate(&e1));
  ED_CUDA(cudaEventRecord(e0, ctx->stream));
  int rc = launch_hv_dispatch(h, x, y);
  ED_CUDA(cudaEventRecord(e1, ctx->stream));
  ctx->prof_events.push_back(e0);
  ctx->prof_events.push_back(e1);
  return rc;
}

int ed_launch_hv_dot(ed_ham* h, const double2* x, double2* y, double2* dot, double* y2) {
  return ed_launch_hv_dot_any(h, x, y, false, dot, y2);
}

int ed_launch_hv_dot_any(ed_ham* h, const void* x, void* y, bool rio, double2* dot, double* y2) {
  ed_ctx* ctx = h->ctx;
  if (!ed_lin_supported(h)) return ED_ENOTSUP;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ctx->profiling) {
    ED_CUDA(cudaEventCreate(&e0));
    ED_CUDA(cudaEventCreate(&e1));
    ED_CUDA(cudaEventRecord(e0, ctx->stream));
  }
  int nblk = 0;
  ED_TRY(ed_launch_hv_lin(h, x, y, true, &nblk, rio));
  if (ctx->profiling) {
    ED_CUDA(cudaEventRecord(e1, ctx->stream));
    ctx->prof_events.push_back(e0);
    ctx->prof_events.push_back(e1);
  }
  double out[3];
  ED_TRY(ed_finish_reduce(ctx, 3, nblk, out));
  dot->x = out[0];
  dot->y = out[1];
  if (y2) *y2 = out[2];
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Explicit CSR: count, scan, fill (columns sorted per row as PETSc AIJ keeps
// them; the values are real because H is real symmetric).
// ---------------------------------------------------------------------------
struct UniqueBonds {
  int n;
  uint32_t mask[ED_MAX_BONDS];
  double val[ED_MAX_BONDS];
};

template <int K>
__global__ void k_csr_count(const uint32_t* __restrict__ states, int64_t dim, const DiagParams dp, const UniqueBonds ub,
                            int64_t* __restrict__ counts) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    uint32_t s = states[r];
    bool he;
    (void)ed_diag_value(s, dp, &he);
    int64_t c = he ? 1 : 0;
    for (int b = 0; b < ub.n; ++b) {
      uint32_t t = s & ub.mask[b];
      if (t != 0u && t != ub.mask[b]) ++c;
    }
    counts[r] = c;
  }
}

template <int K>
__global__ void k_csr_fill(const uint32_t* __restrict__ states, int64_t dim, const DiagParams dp, const UniqueBonds ub,
                           const RankTables rt, const int64_t* __restrict__ rowptr, uint32_t* __restrict__ cols,
                           double* __restrict__ vals) {
  extern __shared__ uint32_t stab[];
  ed_load_tables(stab, rt);
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    uint32_t s = states[r];
    bool he;
    double dv = ed_diag_value(s, dp, &he);
    int64_t o = rowptr[r], n = 0;
    if (he) { cols[o] = (uint32_t)r; vals[o] = dv; n = 1; }
    for (int b = 0; b < ub.n; ++b) {
      uint32_t t = s & ub.mask[b];
      if (t != 0u && t != ub.mask[b]) {
        uint32_t c = ed_rank<K>(s ^ ub.mask[b], stab, rt);
        double v = ub.val[b];
        // insertion into the sorted row segment
        int64_t k = n;
        while (k > 0 && cols[o + k - 1] > c) { cols[o + k] = cols[o + k - 1]; vals[o + k] = vals[o + k - 1]; --k; }
        cols[o + k] = c; vals[o + k] = v;
        ++n;
      }
    }
  }
}

// Block-wise exclusive scan of counts -> rowptr (rowptr has dim+1 entries).
__global__ void k_scan_blocks(const int64_t* __restrict__ in, int64_t n, int64_t per_block, int64_t* __restrict__ sums) {
  int64_t beg = (int64_t)blockIdx.x * per_block, end = min(n, beg + per_block);
  __shared__ int64_t sh[256];
  int64_t acc = 0;
  for (int64_t i = beg + threadIdx.x; i < end; i += blockDim.x) acc += in[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = sh[0];
}

__global__ void k_scan_apply(const int64_t* __restrict__ in, int64_t n, int64_t per_block,
                             const int64_t* __restrict__ offsets, int64_t* __restrict__ out) {
  // serial within the block's chunk, chunked by warps for moderate speed
  if (threadIdx.x != 0) return;
  int64_t beg = (int64_t)blockIdx.x * per_block, end = min(n, beg + per_block);
  int64_t acc = offsets[blockIdx.x];
  for (int64_t i = beg; i < end; ++i) { out[i] = acc; acc += in[i]; }
  if (end == n) out[n] = acc;
}

template <int K>
static int csr_build_k(ed_ham* h) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  DiagParams dp;
  make_diag_params(h, dp);
  UniqueBonds ub;
  memset(&ub, 0, sizeof(ub));
  std::vector<uint32_t> masks;
  std::vector<double> vals;
  ed_ham_unique_masks(h, masks, vals);
  ub.n = (int)masks.size();
  for (int i = 0; i < ub.n; ++i) { ub.mask[i] = masks[i]; ub.val[i] = vals[i]; }
  const int64_t dim = b->dim;
  int64_t* counts = nullptr;
  ED_CUDA(cudaMalloc(&counts, sizeof(int64_t) * (size_t)dim));
  if (!h->d_rowptr) ED_CUDA(cudaMalloc(&h->d_rowptr, sizeof(int64_t) * (size_t)(dim + 1)));
  k_csr_count<K><<<grid_cap(ctx, dim, 256, 8), 256, 0, ctx->stream>>>(b->d_states, dim, dp, ub, counts);
  ED_CHECK_LAUNCH(ctx);
  const int nblk = std::max(1, std::min<int>(4096, (int)((dim + 4095) / 4096)));
  const int64_t per_block = (dim + nblk - 1) / nblk;
  int64_t* sums = nullptr;
  ED_CUDA(cudaMalloc(&sums, sizeof(int64_t) * nblk));
  k_scan_blocks<<<nblk, 256, 0, ctx->stream>>>(counts, dim, per_block, sums);
  ED_CHECK_LAUNCH(ctx);
  std::vector<int64_t> hs(nblk), ho(nblk);
  ED_CUDA(cudaMemcpyAsync(hs.data(), sums, sizeof(int64_t) * nblk, cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  int64_t acc = 0;
  for (int i = 0; i < nblk; ++i) { ho[i] = acc; acc += hs[i]; }
  ED_CUDA(cudaMemcpyAsync(sums, ho.data(), sizeof(int64_t) * nblk, cudaMemcpyHostToDevice, ctx->stream));
  k_scan_apply<<<nblk, 32, 0, ctx->stream>>>(counts, dim, per_block, sums, h->d_rowptr);
  ED_CHECK_LAUNCH(ctx);
  const int64_t nnz = acc;
  if (h->d_cols) { cudaFree(h->d_cols); h->d_cols = nullptr; }
  if (h->d_vals) { cudaFree(h->d_vals); h->d_vals = nullptr; }
  cudaError_t e1 = cudaMalloc(&h->d_cols, sizeof(uint32_t) * (size_t)std::max<int64_t>(nnz, 1));
  cudaError_t e2 = cudaMalloc(&h->d_vals, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaGetLastError();
    cudaFree(counts); cudaFree(sums);
    return ed_fail(ED_ENOMEM, "explicit CSR does not fit in device memory");
  }
  size_t smem = (size_t)b->rt.total * sizeof(uint32_t);
  ED_CUDA(cudaFuncSetAttribute(k_csr_fill<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(56 * 1024)));
  k_csr_fill<K><<<grid_cap(ctx, dim, 128, 8), 128, smem, ctx->stream>>>(b->d_states, dim, dp, ub, b->rt, h->d_rowptr,
                                                                         h->d_cols, h->d_vals);
  ED_CHECK_LAUNCH(ctx);
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(counts);
  cudaFree(sums);
  h->nnz = nnz;
  return ED_OK;
}

int ed_launch_csr_build(ed_ham* h) {
  switch (h->basis->rt.K) {
    case 1: return csr_build_k<1>(h);
    case 2: return csr_build_k<2>(h);
    case 3: return csr_build_k<3>(h);
    default: return csr_build_k<4>(h);
  }
}

// CSR SpMV with 8 lanes per row (4 rows per warp).  The row loop is
// warp-uniform so every lane reaches the shuffles.
__global__ void __launch_bounds__(256) k_csr_spmv(const int64_t* __restrict__ rowptr, const uint32_t* __restrict__ cols,
                                                  const double* __restrict__ vals, const double2* __restrict__ x,
                                                  double2* __restrict__ y, int64_t dim) {
  const int lane8 = threadIdx.x & 7;
  const int sub = (threadIdx.x & 31) >> 3;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r0 = warp * 4; r0 < dim; r0 += nwarps * 4) {
    const int64_t r = r0 + sub;
    const bool valid = r < dim;
    const int64_t b = valid ? rowptr[r] : 0, e = valid ? rowptr[r + 1] : 0;
    double ar = 0.0, ai = 0.0;
    for (int64_t k = b + lane8; k < e; k += 8) {
      const double v = vals[k];
      const double2 xv = __ldg(&x[cols[k]]);
      ar = fma(v, xv.x, ar);
      ai = fma(v, xv.y, ai);
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      ar += __shfl_down_sync(0xffffffffu, ar, o, 8);
      ai += __shfl_down_sync(0xffffffffu, ai, o, 8);
    }
    if (valid && lane8 == 0) y[r] = make_double2(ar, ai);
  }
}

int ed_launch_csr_spmv(ed_ham* h, const double2* x, double2* y) {
  ed_ctx* ctx = h->ctx;
  const int64_t dim = h->basis->dim;
  k_csr_spmv<<<grid_cap(ctx, dim * 8, 256, 8), 256, 0, ctx->stream>>>(h->d_rowptr, h->d_cols, h->d_vals, x, y, dim);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

// ---------------------------------------------------------------------------
// H.v without any device allocation.
//
// ed_ham_apply keeps its quantised copy of x in buffers it allocates on first
// use.  Some callers cannot let a library call cudaMalloc: code that runs
// under a host framework which owns the whole device memory pool, or a
// latency-critical loop that cannot afford the implicit device
// synchronisation an allocation may bring.  ed_ham_apply_noalloc runs the
// same fixed-point H.v (quantise, then gather with exact int64 sums) but keeps
// its scratch in the file-scope array below, which the CUDA module reserves
// when it is loaded, so the call itself allocates nothing.  It is limited to
// ED_NOALLOC_MAX_STATES basis states.
//
// Layout of the scratch array: the first 256 bytes hold the largest exponent
// and the non-finite flag (cleared at every call); the quantised input
// (16 bytes per state) follows.  Every call shares this one array, so calls
// that overlap on the GPU (different streams, or different host threads)
// race on it; the caller must order them.
// ---------------------------------------------------------------------------
#define ED_NOALLOC_HEADER_BYTES 256
static __device__ __align__(256) unsigned char g_noalloc_scratch[ED_NOALLOC_HEADER_BYTES +
                                                                  (size_t)ED_NOALLOC_MAX_STATES * sizeof(longlong2)];

static std::mutex g_noalloc_mutex;
// Per device: the context the address was looked up in, and the address.  A
// device reset (cudaDeviceReset, or a host framework resetting the primary
// context) gives the device a new context and the array a new address, so the
// cached one is used only while the current context is the one it came from.
static void* g_noalloc_ctx[64] = {nullptr};
static void* g_noalloc_ptr[64] = {nullptr};

// The driver's cuCtxGetCurrent, through the runtime (the library does not
// link libcuda); nullptr where the driver does not provide it.
typedef int (*ed_cu_ctx_get_current_t)(void**);
static ed_cu_ctx_get_current_t noalloc_ctx_getter() {
  static ed_cu_ctx_get_current_t fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (ed_cu_ctx_get_current_t)p;
  }
  return fn;
}

// Device address of the scratch array on the current device (the host-side
// symbol is not a device address): looked up with cudaGetSymbolAddress the
// first time on each device, and again whenever the device's current context
// differs from the one of the cached address.
static int noalloc_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= 64) return ed_fail(ED_ENOTSUP, "device index above 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  void* cur = nullptr;
  ed_cu_ctx_get_current_t get = noalloc_ctx_getter();
  if (get && get(&cur) != 0) cur = nullptr;
  if (!g_noalloc_ptr[device] || (cur && cur != g_noalloc_ctx[device])) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return ed_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
    if (get && get(&cur) != 0) cur = nullptr;  // the lookup may have made the primary context current
    g_noalloc_ptr[device] = p;
    g_noalloc_ctx[device] = cur;
  }
  *out = (unsigned char*)g_noalloc_ptr[device];
  return ED_OK;
}

template <int K>
static int launch_hv_noalloc_k(ed_ham* h, const double2* x, double2* y, unsigned char* scratch) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  int* gmax = (int*)scratch;
  longlong2* xq = (longlong2*)(scratch + ED_NOALLOC_HEADER_BYTES);
  int head = 0;
  while ((1 << head) < max_type_count(h->bs) + 1) ++head;
  const int sbits = 62 - head;
  ED_CUDA(cudaMemsetAsync(gmax, 0, 2 * sizeof(int), ctx->stream));
  const int g = grid_cap(ctx, b->dim, 256, 8);
  k_max_exponent<<<g, 256, 0, ctx->stream>>>(x, b->dim, gmax, gmax + 1, nullptr);
  ED_CHECK_LAUNCH(ctx);
  k_quantize64<<<g, 256, 0, ctx->stream>>>(x, b->dim, gmax, sbits, xq, nullptr);
  ED_CHECK_LAUNCH(ctx);
  size_t smem = (size_t)b->rt.total * sizeof(uint32_t);
  ED_CUDA(cudaFuncSetAttribute(k_hv_fx64<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(56 * 1024)));
  int per_sm = 0;
  ED_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_fx64<K>, 256, smem));
  if (per_sm < 1) per_sm = 1;
  k_hv_fx64<K><<<grid_cap(ctx, b->dim, 256, per_sm), 256, smem, ctx->stream>>>(
      b->d_states, h->d_diag, x, xq, gmax, sbits, y, b->dim, b->rt, h->segs, h->bs.chalf[0], h->bs.chalf[1]);
  ED_CHECK_LAUNCH(ctx);
  return ED_OK;
}

extern "C" int ed_ham_apply_noalloc(ed_ham* h, const ed_cplx* x_dev, ed_cplx* y_dev) {
  if (!h || !x_dev || !y_dev) return ed_fail(ED_EINVAL, "null argument");
  if ((const void*)x_dev == (const void*)y_dev) return ed_fail(ED_EINVAL, "x and y must not alias");
  if (h->per_bond) return ed_fail(ED_ENOTSUP, "ed_ham_apply_noalloc supports uniform J1/J2 couplings only");
  if (h->basis->dim > (int64_t)ED_NOALLOC_MAX_STATES)
    return ed_fail(ED_EINVAL, "ed_ham_apply_noalloc handles at most " + std::to_string((long long)ED_NOALLOC_MAX_STATES) +
                                  " basis states; this basis has " + std::to_string((long long)h->basis->dim));
  ED_CUDA(cudaSetDevice(h->ctx->device));
  unsigned char* scratch = nullptr;
  ED_TRY(noalloc_scratch(h->ctx->device, &scratch));
  const double2* x = (const double2*)x_dev;
  double2* y = (double2*)y_dev;
  switch (h->basis->rt.K) {
    case 1: return launch_hv_noalloc_k<1>(h, x, y, scratch);
    case 2: return launch_hv_noalloc_k<2>(h, x, y, scratch);
    case 3: return launch_hv_noalloc_k<3>(h, x, y, scratch);
    default: return launch_hv_noalloc_k<4>(h, x, y, scratch);
  }
}
