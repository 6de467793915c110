// Exact-slice tensor-core contractions (tcgen05) for the real-storage
// Krylov-Schur solve.
//
// GB300 runs FP64 FMA at a small fraction of its tensor rate, and the dense
// tall-skinny contractions of the eigensolve are bound by it.  These kernels
// move the products onto the 5th-generation tensor cores without giving up
// FP64 accuracy: every operand is put in 63-bit fixed point and split into
// eight signed 8-bit slices, which FP16 holds exactly; slice products are
// exact in the tensor core's FP32 accumulator as long as each sum stays
// below 2^24; the sums of equal weight ("levels") are combined in integer
// registers and the result is rounded once to FP64.
//
// Restart combination  out_c = sum_i V_i Y[i][c]  (BVMultInPlace in SLEPc's
// Krylov-Schur restart), for a group of up to 8 outputs:
//  * V (m columns, double[n] each) in tiles of 128 rows.  A tile's entries
//    share one scale 2^P > max |v| (P from the largest exponent among the
//    tile's finite entries): q = round(|v| 2^(63-P)) < 2^63, slices
//    b_s = byte (7-s) of q, s = 0..7, signed like v.
//  * Y column c with its own scale 2^F_c > max_i |Y[i][c]|, slices d_t the
//    same way (built on the host).
//  * One tcgen05.mma chain per tile: D[r][u*8+c] = sum_i sum_{s+t=u} b_s d_t,
//    M = 128 rows (TMEM lanes), K = 8 m (column-major slices), N = 80
//    (levels u = 0..8 for 8 outputs, plus zero padding).  Each D is an
//    integer of magnitude < m * 8 * 255^2 <= 2^24 (m <= 32): exact in FP32.
//  * Epilogue (one thread per row): T_c = sum_u D_u 2^(8(8-u)) exactly in
//    128-bit integers, out = T_c 2^(P + F_c - 78) rounded once to FP64 with
//    integer operations only (the FP64 unit is what this path avoids).
//  * Accuracy: the dropped levels u >= 9 and the two quantisations are below
//    m * 2^-61 of 2^(P + F_c), against FP64 FMA's 16 roundings of 2^-53 of
//    the partial sums.  A row holding a non-finite entry gives NaN outputs;
//    results below 2^-1022 flush to zero.
//
// Requirements: m <= 32, nc <= 8, one GPU.  Persistent grid; each CTA
// pipelines its tiles across loader, MMA and epilogue warps through two
// shared-memory stages and two TMEM accumulators (256 columns per CTA).
// Every wait is bounded: after 2^26 polls the kernel sets an error flag,
// waits (again bounded) for its own MMAs, frees its TMEM and returns; the
// host turns the flag into ED_ECUDA.
#include "ed_internal.h"
#include "ed_device.cuh"
#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int TC_ROWS = 128;        // M: rows per tile = TMEM lanes
constexpr int TC_N = 80;            // N: 9 levels x 8 outputs, padded to a multiple of 16
constexpr int TC_LEVELS = 9;
constexpr int TC_MAX_COLS = 32;     // m <= 32 keeps every level sum below 2^24
constexpr long long TC_WAIT_POLLS = 1ll << 26;

struct TcCols {
  const double* p[TC_MAX_COLS];
};
struct TcOut {
  double* p[8];
  int F[8];  // per-output scale exponents of Y
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor, K-major operand without swizzle:
// 8-row x 16-byte core matrices, lbo = bytes between core matrices adjacent
// in K, sbo = bytes between core matrices adjacent in M/N.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
  return d;                // base offset 0, layout: no swizzle
}

// Instruction descriptor of tcgen05.mma kind::f16: FP16 A and B (K-major),
// FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, long long polls) {
  for (long long k = 0; k < polls; ++k) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Two FP16 slices from bytes (hi, lo) of a 32-bit word: PRMT places each byte
// under the exponent of 1024, an FP16 FMA removes the 1024 and applies the
// sign (exact: operands and results are integers below 2048).
__device__ __forceinline__ uint32_t slice_pair(uint32_t w, uint32_t sel, __half2 sgn, __half2 off) {
  uint32_t x;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(x) : "r"(w), "r"(0x64646464u), "r"(sel));
  __half2 h = __hfma2(*reinterpret_cast<__half2*>(&x), sgn, off);
  return *reinterpret_cast<uint32_t*>(&h);
}

// q = round(|v| 2^(63 - P)) for a tile whose largest biased exponent is E
// (P = E - 1022, so q < 2^63); 0 for zeros, subnormals and non-finite v.
__device__ __forceinline__ unsigned long long fx63(unsigned long long bits, int E) {
  const int e = (int)((bits >> 52) & 0x7FF);
  if (e == 0 || e == 0x7FF) return 0ull;
  const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = e - E + 10;  // <= 10
  if (sh >= 0) return mant << sh;
  if (sh > -64) return (mant + (1ull << (-sh - 1))) >> (-sh);
  return 0ull;
}

// Eight rows' slices, transposed and stored: slice s of rows 0..7 as eight
// FP16 values (16 bytes, the row-contiguous order of a K-major core-matrix
// row) at dst + 16 s.  bits[k]: FP64 bits of row k; E: the scale's exponent.
__device__ __forceinline__ void slices8_store(const unsigned long long (&bits)[8], int E, unsigned char* dst) {
  const __half2 one2 = __floats2half2_rn(1.0f, 1.0f), mone2 = __floats2half2_rn(-1.0f, -1.0f);
  const __half2 offp = __floats2half2_rn(-1024.0f, -1024.0f), offn = __floats2half2_rn(1024.0f, 1024.0f);
  uint32_t P[8][4];  // row k: slice pairs (0,1), (2,3), (4,5), (6,7)
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const unsigned long long q = fx63(bits[k], E);
    const bool ng = (bits[k] >> 63) != 0ull;
    const __half2 sg = ng ? mone2 : one2, of = ng ? offn : offp;
    const uint32_t qh = (uint32_t)(q >> 32), ql = (uint32_t)q;
    P[k][0] = slice_pair(qh, 0x4243u, sg, of);
    P[k][1] = slice_pair(qh, 0x4041u, sg, of);
    P[k][2] = slice_pair(ql, 0x4243u, sg, of);
    P[k][3] = slice_pair(ql, 0x4041u, sg, of);
  }
#pragma unroll
  for (int sl = 0; sl < 8; ++sl) {
    const uint32_t sel = (sl & 1) ? 0x7632u : 0x5410u;
    uint32_t w0, w1, w2, w3;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(w0) : "r"(P[0][sl >> 1]), "r"(P[1][sl >> 1]), "r"(sel));
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(w1) : "r"(P[2][sl >> 1]), "r"(P[3][sl >> 1]), "r"(sel));
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(w2) : "r"(P[4][sl >> 1]), "r"(P[5][sl >> 1]), "r"(sel));
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(w3) : "r"(P[6][sl >> 1]), "r"(P[7][sl >> 1]), "r"(sel));
    *reinterpret_cast<uint4*>(dst + sl * 16) = make_uint4(w0, w1, w2, w3);
  }
}

// Restart combination, pipelined across warp roles (one CTA loops over its
// tiles t = blockIdx.x + k gridDim.x):
//  * loader warps 0..3 (thread = row): load the row's m entries, the tile
//    scale (largest exponent, over the four warps), the eight slices of
//    each entry into shared stage k % 2, then arrive on full[stage];
//  * warp 8, one thread: wait full[stage] and tempty[acc], issue the MMA
//    chain into TMEM accumulator k % 2, commit to empty[stage] (the stage may
//    be refilled) and tfull[acc];
//  * epilogue warps 4..7 (thread = row = TMEM lane): wait tfull[acc], read
//    the 9 levels of the 8 outputs, arrive on tempty[acc] (the accumulator
//    may be reused), then combine the levels and store.
// The tile scale and the rows' non-finite flags travel in a ring of 4 slots,
// each with an mbarrier the epilogue waits on: a loader writing tile k has
// seen the MMA of tile k - 2 complete, which needed the epilogue of tile
// k - 4 to release its accumulator after reading slot k % 4, so the slot is
// free and its barrier at most one phase ahead.
// Every wait is bounded (TC_WAIT_POLLS polls): on a timeout the role sets
// the error flag and leaves its loop; the other roles then time out too,
// the issuing thread waits (bounded) for its own MMAs, and the TMEM is freed.
constexpr int RS_THREADS = 288;  // loaders 0..3, epilogue 4..7, issuer 8
constexpr int RS_TMEM_COLS = 256;  // two accumulators of TC_N columns

struct RsShared {
  uint64_t full[2], empty[2], tfull[2], tempty[2], meta[4], done;
  uint32_t tmem;
  int wmax[2][4];
  uint32_t wbad[2][4];
  int ok[2];
  int E[4];
  uint32_t bad[4][4];
};

template <int MAXC>
__global__ void __launch_bounds__(RS_THREADS) k_restart_tc(const TcCols cols, int m, int kp, const uint4* __restrict__ Bg,
                                                           TcOut out, int nc, int64_t n, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ RsShared S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kgroups = kp / 8;
  const uint32_t a_lbo = (TC_ROWS / 8) * 128, b_lbo = (TC_N / 8) * 128;
  const size_t a_bytes = (size_t)kgroups * a_lbo;
  unsigned char* sB = tc_smem;
  unsigned char* sA0 = tc_smem + (size_t)kgroups * b_lbo;  // stage st at sA0 + st * a_bytes
  {
    const int nvec = kgroups * (TC_N / 8) * 8;  // 16-byte rows of B
    for (int k = tid; k < nvec; k += RS_THREADS) reinterpret_cast<uint4*>(sB)[k] = Bg[k];
    if (kp > 8 * m)  // the zero padding column of A, in both stages
      for (int r = tid; r < 2 * TC_ROWS; r += RS_THREADS)
        *reinterpret_cast<uint4*>(sA0 + (size_t)(r / TC_ROWS) * a_bytes + (size_t)m * a_lbo + ((r % TC_ROWS) >> 3) * 128 +
                                  (r & 7) * 16) =
            make_uint4(0, 0, 0, 0);
  }
  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                 "r"(RS_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&S.full[i])), "r"(128));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.empty[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.tfull[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&S.tempty[i])), "r"(128));
    }
    for (int i = 0; i < 4; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.meta[i])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.done)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B and the padding, for the tensor core
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = S.tmem;
  const int64_t ntiles = (n + TC_ROWS - 1) / TC_ROWS;
  if (warp < 4) {
    // ---------------- loaders ----------------
    const __half2 one2 = __floats2half2_rn(1.0f, 1.0f), mone2 = __floats2half2_rn(-1.0f, -1.0f);
    const __half2 offp = __floats2half2_rn(-1024.0f, -1024.0f), offn = __floats2half2_rn(1024.0f, 1024.0f);
    int k = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int st = k & 1, ring = k & 3;
      const int64_t row = t * TC_ROWS + tid;
      const bool valid = row < n;
      double v[MAXC];
      int emax = 0;
      bool bad = false;
#pragma unroll
      for (int i = 0; i < MAXC; ++i) {
        if (i < m) {
          v[i] = valid ? __ldg(cols.p[i] + row) : 0.0;
          const int e = (int)((__double_as_longlong(v[i]) >> 52) & 0x7FF);
          if (e == 0x7FF) bad = true; else emax = max(emax, e);
        }
      }
      emax = __reduce_max_sync(0xFFFFFFFFu, (unsigned)emax);
      const uint32_t badw = __ballot_sync(0xFFFFFFFFu, bad);
      if (lane == 0) {
        S.wmax[k & 1][warp] = emax;
        S.wbad[k & 1][warp] = badw;
      }
      // one thread waits for the stage, so every loader takes the same branch
      if (tid == 0) S.ok[k & 1] = mbar_wait(smem_u32(&S.empty[st]), ((k >> 1) & 1) ^ 1, TC_WAIT_POLLS) ? 1 : 0;
      asm volatile("bar.sync 1, 128;" ::: "memory");
      if (!S.ok[k & 1]) {
        if (tid == 0) atomicExch(err, 1);
        break;
      }
      const int E = max(max(S.wmax[k & 1][0], S.wmax[k & 1][1]), max(S.wmax[k & 1][2], S.wmax[k & 1][3]));
      if (tid == 0) {  // the tile's scale and non-finite rows for the epilogue
        S.E[ring] = E;
        for (int q = 0; q < 4; ++q) S.bad[ring][q] = S.wbad[k & 1][q];
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&S.meta[ring])) : "memory");
      }
      unsigned char* a = sA0 + (size_t)st * a_bytes;
#pragma unroll
      for (int i = 0; i < MAXC; ++i) {
        if (i < m) {
          const unsigned long long bits = (unsigned long long)__double_as_longlong(v[i]);
          const unsigned long long q = fx63(bits, E);
          const bool ng = (bits >> 63) != 0ull;
          const __half2 sg = ng ? mone2 : one2, of = ng ? offn : offp;
          const uint32_t qh = (uint32_t)(q >> 32), ql = (uint32_t)q;
          uint4 w;
          w.x = slice_pair(qh, 0x4243u, sg, of);  // slices 0, 1 (bytes 7, 6 of q)
          w.y = slice_pair(qh, 0x4041u, sg, of);  // slices 2, 3
          w.z = slice_pair(ql, 0x4243u, sg, of);  // slices 4, 5
          w.w = slice_pair(ql, 0x4041u, sg, of);  // slices 6, 7
          *reinterpret_cast<uint4*>(a + (size_t)i * a_lbo + (tid >> 3) * 128 + (tid & 7) * 16) = w;
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&S.full[st])) : "memory");
    }
  } else if (warp < 8) {
    // ---------------- epilogue ----------------
    const int r = tid - 128;  // TMEM lane
    int k = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int ac = k & 1, ring = k & 3;
      if (!mbar_wait(smem_u32(&S.tfull[ac]), (k >> 1) & 1, TC_WAIT_POLLS) ||
          !mbar_wait(smem_u32(&S.meta[ring]), (k >> 2) & 1, TC_WAIT_POLLS)) {
        atomicExch(err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      // read the ring before releasing the accumulator: once it is released,
      // the loaders may reach tile k + 4 and refill slot k % 4
      const int P = S.E[ring] - 1022;
      const bool bad = (S.bad[ring][r >> 5] >> (r & 31)) & 1u;
      long long Ah[8], Bl[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) Ah[c] = Bl[c] = 0;
      const uint32_t taddr = tmem + ((uint32_t)((warp - 4) * 32) << 16) + (uint32_t)(ac * 128);
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        uint32_t d[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7]),
              "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]), "=r"(d[14]), "=r"(d[15])
            : "r"(taddr + (uint32_t)(16 * j)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int u = 2 * j + h;
          if (u < TC_LEVELS) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
              const long long dv = (long long)__float2int_rz(__uint_as_float(d[h * 8 + c]));
              if (u < 4) Ah[c] = Ah[c] * 256 + dv;
              else Bl[c] = Bl[c] * 256 + dv;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&S.tempty[ac])) : "memory");
      const int64_t row = t * TC_ROWS + r;
      if (row < n) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          if (c < nc) {
            long long hi = Ah[c] >> 24;
            unsigned long long lo = (unsigned long long)Ah[c] << 40;
            const unsigned long long lo2 = lo + (unsigned long long)Bl[c];
            hi += (Bl[c] >> 63) + (lo2 < lo ? 1ll : 0ll);
            double x = ed_fx128_to_double(hi, lo2, P + out.F[c] - 78);
            if (bad) x = __longlong_as_double(0x7FF8000000000000ll);
            out.p[c][row] = x;
          }
        }
      }
    }
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = umma_idesc_f16(TC_ROWS, TC_N);
    const uint32_t b_base = smem_u32(sB);
    int k = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
      const int st = k & 1, ac = k & 1;
      if (!mbar_wait(smem_u32(&S.full[st]), (k >> 1) & 1, TC_WAIT_POLLS) ||
          !mbar_wait(smem_u32(&S.tempty[ac]), ((k >> 1) & 1) ^ 1, TC_WAIT_POLLS)) {
        atomicExch(err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a_base = smem_u32(sA0 + (size_t)st * a_bytes);
      for (int ks = 0; ks < kp / 16; ++ks) {
        const uint64_t ad = umma_desc(a_base + ks * 2 * a_lbo, a_lbo, 128);
        const uint64_t bd = umma_desc(b_base + ks * 2 * b_lbo, b_lbo, 128);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem + (uint32_t)(ac * 128)),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&S.empty[st]))
                   : "memory");
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&S.tfull[ac]))
                   : "memory");
    }
    // every MMA this thread issued has completed before the TMEM is freed
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(&S.done))
                 : "memory");
    if (!mbar_wait(smem_u32(&S.done), 0, TC_WAIT_POLLS)) atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 8) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(RS_TMEM_COLS));
}

// Dot products h_i = V_i^T w for up to 16 columns on the tensor cores, in
// exact slices.  Per 128-row tile: w (after the local Lanczos step
// w <- w - a vj - b vjm1 when LOCAL, written back in FP64) and every column
// get their own scale (largest exponent in the tile), eight signed 8-bit
// slices of 63-bit fixed point each; one tcgen05.mma chain gives
// D[(i, s)][t] = sum_rows b_s(v_i) d_t(w) exactly (M = 128 = 16 columns x 8
// slices, N = 16 (8 used), K = 128 rows; |D| < 128 x 255^2 < 2^23).  TMEM
// lane (i, s) adds X = sum_t D_t 2^(8(7-t)) for every tile into an exact
// 128-bit accumulator at the unit 2^(Pref + Qref - 126), shifted by the tile
// scales relative to Pref = 1 (|v| <= 1) and Qref (a bound on max |w| from
// the host); a tile more than 2^-40 below the reference contributes with a
// rounding of half a unit (2^-127 of the reference scale).  Each CTA rounds
// lane by lane to FP64 and sums the 8 slices of a column in fixed order into
// its partial; the partials are summed like every other reduction.
constexpr int DT_THREADS = 256;
constexpr int DT_COLS = 16;
constexpr int DT_N = 16;
constexpr int DT_TMEM_COLS = 32;

struct DotCols {
  const double* p[DT_COLS];
};

template <bool LOCAL>
__global__ void __launch_bounds__(DT_THREADS) k_dots_tc(const __grid_constant__ DotCols cols, int ng, double* __restrict__ w,
                                                        const double* __restrict__ vj, double a,
                                                        const double* __restrict__ vjm1, double b, int qref,
                                                        int64_t n, unsigned long long* __restrict__ part,
                                                        int* __restrict__ err) {
  __shared__ __align__(1024) unsigned char sA[16 * 16 * 128];  // [rg][i][s][row] halves
  __shared__ __align__(1024) unsigned char sB[16 * 2 * 128];   // [rg][t-group][t][row] halves
  __shared__ uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_P[DT_COLS];
  __shared__ int s_Q;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // zero the unused half of B (slices t = 8..15) and the columns i >= ng of A
  for (int k = tid; k < 16 * 8; k += DT_THREADS) {
    *reinterpret_cast<uint4*>(sB + (k >> 3) * 256 + 128 + (k & 7) * 16) = make_uint4(0, 0, 0, 0);
  }
  for (int k = tid; k < 16 * 16 * 8; k += DT_THREADS) {
    const int i = (k >> 3) & 15;
    if (i >= ng) *reinterpret_cast<uint4*>(sA + (k >> 7) * 2048 + i * 128 + (k & 7) * 16) = make_uint4(0, 0, 0, 0);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(DT_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;
  const uint32_t bar = smem_u32(&s_bar);
  const uint32_t idesc = umma_idesc_f16(128, DT_N);
  const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
  const int ci = tid >> 4, rg = tid & 15;  // this thread's column and 8-row group
  // drain lanes: warps 0..3, TMEM lane = tid = i * 8 + s
  const int di = tid >> 3;
  long long acc_hi = 0;
  unsigned long long acc_lo = 0;
  const int64_t ntiles = (n + 127) / 128;
  uint32_t phase = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t r0 = t * 128 + rg * 8;
    // w task (threads 0..15): the local step, then the tile scale of w
    unsigned long long wb[8];
    if (tid < 16) {
      int e = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t r = r0 + k;
        double x = 0.0;
        if (r < n) {
          x = w[r];
          if (LOCAL) {
            x = fma(-a, vj[r], x);
            if (vjm1) x = fma(-b, vjm1[r], x);
            w[r] = x;
          }
        }
        wb[k] = (unsigned long long)__double_as_longlong(x);
        const int ex = (int)((wb[k] >> 52) & 0x7FF);
        if (ex != 0x7FF) e = max(e, ex);
      }
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0x0000FFFFu, e, o, 16));
      if (tid == 0) s_Q = e;
      slices8_store(wb, e, sB + rg * 256);
    }
    // V tasks: column ci, rows r0..r0+7
    if (ci < ng) {
      unsigned long long vb[8];
      int e = 0;
      const double* col = cols.p[ci];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t r = r0 + k;
        const double x = r < n ? __ldg(col + r) : 0.0;
        vb[k] = (unsigned long long)__double_as_longlong(x);
        const int ex = (int)((vb[k] >> 52) & 0x7FF);
        if (ex != 0x7FF) e = max(e, ex);
      }
      const unsigned mask = (lane < 16) ? 0x0000FFFFu : 0xFFFF0000u;
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(mask, e, o, 16));
      if (rg == 0) s_P[ci] = e;
      slices8_store(vb, e, sA + rg * 2048 + ci * 128);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int ks = 0; ks < 8; ++ks) {
        const uint64_t ad = umma_desc(a_base + ks * 2 * 2048, 2048, 128);
        const uint64_t bd = umma_desc(b_base + ks * 2 * 256, 256, 128);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                   : "memory");
    }
    const bool done = mbar_wait(bar, phase, TC_WAIT_POLLS);
    if (!__syncthreads_and(done)) {
      if (tid == 0) atomicExch(err, 1);
      mbar_wait(bar, phase, TC_WAIT_POLLS);
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp < 4) {
      uint32_t d[8];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
          : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16)));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (di < ng) {
        long long H = 0, L = 0;
#pragma unroll
        for (int q = 0; q < 5; ++q) H = H * 256 + (long long)__float2int_rz(__uint_as_float(d[q]));
#pragma unroll
        for (int q = 5; q < 8; ++q) L = L * 256 + (long long)__float2int_rz(__uint_as_float(d[q]));
        // X = H 2^24 + L as 128 bits
        long long xh = H >> 40;
        unsigned long long xl = (unsigned long long)H << 24;
        const unsigned long long xl2 = xl + (unsigned long long)L;
        xh += (L >> 63) + (xl2 < xl ? 1ll : 0ll);
        xl = xl2;
        // (Pref - P) + (Qref - Q) with biased tile exponents; Pref = 1
        const int sh = (1 - s_P[di]) + (qref - s_Q) + 1022;
        if (sh < 0) atomicExch(err, 2);  // w above the host's bound: the host redoes the pass in FP64
        if (sh >= 0 && sh < 100) {
          if (sh > 0 && sh <= 63) {  // arithmetic shift of the 128-bit X, rounding half up
            const unsigned long long l2 = xl + (1ull << (sh - 1));
            xh += l2 < xl ? 1ll : 0ll;
            xl = (l2 >> sh) | ((unsigned long long)xh << (64 - sh));
            xh >>= sh;
          } else if (sh >= 64) {
            if (sh == 64) {
              const unsigned long long l2 = xl + (1ull << 63);
              xh += l2 < xl ? 1ll : 0ll;
            } else {
              xh += 1ll << (sh - 65);
            }
            xl = (unsigned long long)(xh >> (sh - 64));
            xh >>= 63;
          }
          const unsigned long long l2 = acc_lo + xl;
          acc_hi += xh + (l2 < acc_lo ? 1ll : 0ll);
          acc_lo = l2;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
    }
    __syncthreads();
  }
  // lane (i, s): acc at the unit 2^(8(7-s)) 2^(Pref + Qref - 126), Pref = 1;
  // the exact sum over the CTAs is k_dots_finish's
  if (warp < 4) {
    unsigned long long* dst = part + ((size_t)blockIdx.x * 128 + tid) * 2;
    dst[0] = acc_lo;
    dst[1] = (unsigned long long)acc_hi;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(DT_TMEM_COLS));
}

// Magnitude of a 4-word (256-bit) unsigned integer times 2^X, rounded to
// nearest even, as FP64 with the given sign; integer operations only.
__device__ __forceinline__ double u256_to_double(const unsigned long long (&w)[4], int X, bool neg) {
  int k = 3;
  while (k > 0 && w[k] == 0ull) --k;
  if (w[k] == 0ull) return 0.0;
  const int L = 64 * k + 64 - __clzll((long long)w[k]);  // bit length
  // the top 64 bits (leading bit at 63) and a sticky bit for the rest
  unsigned long long top, rest;
  const int sh = L - 64;  // bits below the top word
  if (sh <= 0) {
    top = w[0] << (-sh);
    rest = 0ull;
  } else {
    const int q = sh >> 6, r = sh & 63;
    top = r ? ((w[q] >> r) | (q + 1 < 4 ? (w[q + 1] << (64 - r)) : 0ull)) : w[q];
    rest = r ? (w[q] & ((1ull << r) - 1ull)) : 0ull;
    for (int j = 0; j < q; ++j) rest |= w[j];
  }
  unsigned long long m = top >> 11;  // 53 bits
  const unsigned long long low = top & 0x7FFull;
  const bool up = low > 0x400ull || (low == 0x400ull && (rest != 0ull || (m & 1ull)));
  m += up ? 1ull : 0ull;
  int bexp = X + L + 1022;
  if (m >> 53) {
    m >>= 1;
    ++bexp;
  }
  if (bexp <= 0) return 0.0;
  const unsigned long long bits =
      ((unsigned long long)neg << 63) | ((unsigned long long)bexp << 52) | (m & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

// Exact sum of the CTAs' lane accumulators of k_dots_tc (thread = lane
// (i, s)), the slices of each column combined with their weights 2^(8(7-s))
// in 256-bit integers, and one rounding per column:
// h[item0 + i] = total_i 2^(Pref + Qref - 126).
__global__ void __launch_bounds__(128) k_dots_finish(const unsigned long long* __restrict__ part, int nblk, int ng,
                                                     int qref, double* __restrict__ h, int item0) {
  __shared__ unsigned long long sh[128][4];
  const int t = threadIdx.x, i = t >> 3, sl = t & 7;
  // 192-bit signed sum of nblk 128-bit values
  unsigned long long a0 = 0ull, a1 = 0ull, a2 = 0ull;
  for (int b = 0; b < nblk; ++b) {
    const unsigned long long lo = part[((size_t)b * 128 + t) * 2];
    const unsigned long long hi = part[((size_t)b * 128 + t) * 2 + 1];
    const unsigned long long ext = (long long)hi < 0 ? ~0ull : 0ull;
    const unsigned long long s0 = a0 + lo;
    const unsigned long long c0 = s0 < a0 ? 1ull : 0ull;
    const unsigned long long s1 = a1 + hi;
    const unsigned long long c1 = s1 < a1 ? 1ull : 0ull;
    const unsigned long long s1b = s1 + c0;
    const unsigned long long c1b = s1b < s1 ? 1ull : 0ull;
    a2 += ext + c1 + c1b;
    a1 = s1b;
    a0 = s0;
  }
  // times 2^(8(7-s)) into 256 bits (sign-extended)
  const int sh8 = 8 * (7 - sl);
  unsigned long long v[4];
  const unsigned long long a3 = (long long)a2 < 0 ? ~0ull : 0ull;
  if (sh8 == 0) {
    v[0] = a0; v[1] = a1; v[2] = a2; v[3] = a3;
  } else {
    v[0] = a0 << sh8;
    v[1] = (a1 << sh8) | (a0 >> (64 - sh8));
    v[2] = (a2 << sh8) | (a1 >> (64 - sh8));
    v[3] = (a3 << sh8) | (a2 >> (64 - sh8));
  }
  for (int k = 0; k < 4; ++k) sh[t][k] = v[k];
  __syncthreads();
  if (sl == 0 && i < ng) {
    unsigned long long w[4] = {0ull, 0ull, 0ull, 0ull};
    for (int q = 0; q < 8; ++q) {
      unsigned long long carry = 0ull;
      for (int k = 0; k < 4; ++k) {
        const unsigned long long x = sh[t + q][k];
        const unsigned long long s1 = w[k] + x;
        const unsigned long long c1 = s1 < w[k] ? 1ull : 0ull;
        const unsigned long long s2 = s1 + carry;
        const unsigned long long c2 = s2 < s1 ? 1ull : 0ull;
        w[k] = s2;
        carry = c1 + c2;
      }
    }
    const bool neg = (long long)w[3] < 0;
    if (neg) {  // two's complement negation
      unsigned long long carry = 1ull;
      for (int k = 0; k < 4; ++k) {
        const unsigned long long x = ~w[k] + carry;
        carry = (carry && x == 0ull) ? 1ull : 0ull;
        w[k] = x;
      }
    }
    h[item0 + i] = u256_to_double(w, 1 + (qref - 1022) - 126, neg);
  }
}

}  // namespace

// CTAs of a tensor-core kernel that fit one SM at once, from its registers,
// shared memory, threads and TMEM columns.  (The occupancy query reports one
// CTA per SM for kernels that allocate tensor memory, which would leave the
// per-tile latency of these kernels exposed.)
template <typename K>
static int tc_ctas_per_sm(K kern, int threads, size_t dyn_smem, int tmem_cols) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  int dev = 0, smem_sm = 0, regs_sm = 0, thr_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  const size_t per_cta_smem = dyn_smem + fa.sharedSizeBytes + 1024;  // + the per-CTA reserve
  int n = 512 / tmem_cols;
  n = std::min(n, (int)((size_t)smem_sm / std::max<size_t>(per_cta_smem, 1)));
  n = std::min(n, thr_sm / threads);
  const int regs = std::max(fa.numRegs, 1) * threads;
  n = std::min(n, regs_sm / regs);
  return std::max(n, 1);
}

// Host: B operand for one group of up to 8 outputs (columns c0..c0+nc-1 of
// Y, row-major ldY), in the shared-memory layout of the kernel, and the
// outputs' scale exponents.
static void tc_build_b(const double* Y, int ldY, int m, int kp, int c0, int nc, std::vector<uint16_t>& B, int F[8]) {
  const int kgroups = kp / 8;
  B.assign((size_t)kgroups * TC_N * 8, 0);
  for (int c = 0; c < 8; ++c) {
    F[c] = 0;
    if (c >= nc) continue;
    double mx = 0.0;
    for (int i = 0; i < m; ++i) mx = std::max(mx, std::fabs(Y[(size_t)i * ldY + c0 + c]));
    int e = 0;
    if (mx > 0.0) std::frexp(mx, &e);  // mx < 2^e
    F[c] = e;
    for (int i = 0; i < m; ++i) {
      const double y = Y[(size_t)i * ldY + c0 + c];
      const unsigned long long q = (unsigned long long)std::llround(std::ldexp(std::fabs(y), 63 - e));
      const bool ng = std::signbit(y);
      for (int u = 0; u < TC_LEVELS; ++u)
        for (int s = 0; s < 8; ++s) {
          const int tq = u - s;
          if (tq < 0 || tq > 7) continue;
          const int d = (int)((q >> (8 * (7 - tq))) & 0xFFull);
          const __half h = __float2half_rn(ng ? -(float)d : (float)d);
          uint16_t hb;
          std::memcpy(&hb, &h, 2);
          const int nrow = u * 8 + c, k = i * 8 + s;
          B[(size_t)(k / 8) * (TC_N / 8) * 64 + (nrow / 8) * 64 + (nrow % 8) * 8 + (k % 8)] = hb;
        }
    }
  }
}

int ed_restart_combine_tc(ed_ctx* ctx, const double* const* cols, int m, const double* Y, int ldY, int l,
                          double* const* out, int64_t n) {
  if (m < 1 || m > TC_MAX_COLS) return ED_ENOTSUP;
  const int kp = ((m + 1) / 2) * 16;
  const int kgroups = kp / 8;
  const size_t smem = (size_t)kgroups * (2 * (TC_ROWS / 8) + TC_N / 8) * 128;  // two A stages and B
  const size_t bwords = (size_t)kgroups * TC_N * 8;  // halves per group
  const int ngroups = (l + 7) / 8;
  ED_TRY(ed_ensure_reduce(ctx, (size_t)ngroups * bwords / 4 + 8));
  uint16_t* dB = (uint16_t*)ctx->d_red;
  int* d_err = (int*)(ctx->d_red + (size_t)ngroups * bwords / 4 + 4);
  std::vector<uint16_t> B, all;
  std::vector<TcOut> outs(ngroups);
  all.reserve((size_t)ngroups * bwords);
  for (int g = 0; g < ngroups; ++g) {
    const int nc = std::min(8, l - g * 8);
    tc_build_b(Y, ldY, m, kp, g * 8, nc, B, outs[g].F);
    all.insert(all.end(), B.begin(), B.end());
    for (int c = 0; c < 8; ++c) outs[g].p[c] = c < nc ? out[g * 8 + c] : nullptr;
  }
  ED_CUDA(cudaMemcpyAsync(dB, all.data(), sizeof(uint16_t) * all.size(), cudaMemcpyHostToDevice, ctx->stream));
  ED_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  auto kern = m <= 16 ? k_restart_tc<16> : k_restart_tc<32>;
  ED_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int per_sm = tc_ctas_per_sm(kern, RS_THREADS, smem, RS_TMEM_COLS);
  const int64_t ntiles = (n + TC_ROWS - 1) / TC_ROWS;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)ctx->num_sms * per_sm));
  TcCols cp;
  for (int i = 0; i < TC_MAX_COLS; ++i) cp.p[i] = i < m ? cols[i] : nullptr;
  for (int g = 0; g < ngroups; ++g) {
    kern<<<grid, RS_THREADS, smem, ctx->stream>>>(cp, m, kp, (const uint4*)(dB + (size_t)g * bwords), outs[g],
                                                  std::min(8, l - g * 8), n, d_err);
    ED_CHECK_LAUNCH(ctx);
  }
  int h_err = 0;
  ED_CUDA(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));  // also keeps the host coefficients alive for the copy
  if (h_err) return ed_fail(ED_ECUDA, "tensor-core restart: completion wait timed out");
  return ED_OK;
}


// h_host[i] = V_i^T w (i < nv) on the tensor cores in exact slices; with vj
// the local step w <- w - a vj - b vjm1 first (written back).  wbound: an
// upper bound on max_r |w_r| after the local step.
int ed_multidot_tc(ed_ctx* ctx, const double* const* cols, int nv, double* w, int64_t n, const double* vj, double a,
                   const double* vjm1, double b, double wbound, double* h_host) {
  if (nv < 1 || nv > 127) return ED_ENOTSUP;
  if (!(wbound > 0.0) || !std::isfinite(wbound)) return ED_ENOTSUP;
  int qe = 0;
  std::frexp(wbound, &qe);  // wbound < 2^qe
  const int qref = qe + 1022;  // biased exponent E with max |w| < 2^(E - 1022)
  const int per_sm = tc_ctas_per_sm(k_dots_tc<false>, DT_THREADS, 0, DT_TMEM_COLS);
  const int64_t ntiles = (n + 127) / 128;
  const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)ctx->num_sms * per_sm));
  const int ngroups = (nv + DT_COLS - 1) / DT_COLS;
  const size_t part_words = (size_t)nblk * 128 * 2;  // per group
  ED_TRY(ed_ensure_reduce(ctx, (size_t)ngroups * part_words + nv + 8));
  unsigned long long* part = (unsigned long long*)ctx->d_red;
  double* h_dev = ctx->d_red + (size_t)ngroups * part_words;
  int* d_err = (int*)(h_dev + nv + 4);
  ED_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  for (int g = 0; g < ngroups; ++g) {
    const int v0 = g * DT_COLS, ng = std::min(DT_COLS, nv - v0);
    DotCols cp;
    for (int i = 0; i < DT_COLS; ++i) cp.p[i] = i < ng ? cols[v0 + i] : nullptr;
    unsigned long long* pg = part + (size_t)g * part_words;
    if (g == 0 && vj)
      k_dots_tc<true><<<nblk, DT_THREADS, 0, ctx->stream>>>(cp, ng, w, vj, a, vjm1, b, qref, n, pg, d_err);
    else
      k_dots_tc<false><<<nblk, DT_THREADS, 0, ctx->stream>>>(cp, ng, w, nullptr, 0.0, nullptr, 0.0, qref, n, pg, d_err);
    ED_CHECK_LAUNCH(ctx);
    k_dots_finish<<<1, 128, 0, ctx->stream>>>(pg, nblk, ng, qref, h_dev, v0);
    ED_CHECK_LAUNCH(ctx);
  }
  // the sums and the error flag in one copy
  ED_CUDA(cudaMemcpyAsync(ctx->h_red, h_dev, sizeof(double) * (nv + 5), cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<double> out(ctx->h_red, ctx->h_red + nv);
  const int h_err = *(const int*)(ctx->h_red + nv + 4);
  if (h_err == 2) return ED_ENOTSUP;  // the bound on max |w| did not hold: nothing wrong, use FP64
  if (h_err) return ed_fail(ED_ECUDA, "tensor-core dot products: completion wait timed out");
  for (int i = 0; i < nv; ++i) h_host[i] = out[i];
  return ED_OK;
}
