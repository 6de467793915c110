// Run-time specialised two-table H.v: the bond masks of one operator become
// immediates of a kernel compiled for it with NVRTC (sm_103a cubin), so each
// bond slot costs only its flip test, one table lookup and the gather (no
// bond-word loads, no loop bookkeeping, all bonds of a row unrolled).  Same
// arithmetic as k_hv_lin (exact int64 sums per coupling type, one rounding),
// so the results are bit-identical; the autotuner in ed_hv_lin.cu times it
// beside the static variants.  NVRTC is loaded with dlopen and the driver
// API through cudaGetDriverEntryPointByVersion, so the library needs neither
// at link time; where either is missing this variant is simply unavailable.
#include "ed_internal.h"
#include <cuda.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <cstdio>
#include <cstdlib>
#include <sys/stat.h>
#include <unistd.h>
#include <algorithm>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#ifndef ED_CUDA_LIB_DIR
#define ED_CUDA_LIB_DIR "/usr/local/cuda/lib64"
#endif

namespace {

struct Nvrtc {
  bool ok = false;
  nvrtcResult (*create)(nvrtcProgram*, const char*, const char*, int, const char* const*, const char* const*) = nullptr;
  nvrtcResult (*compile)(nvrtcProgram, int, const char* const*) = nullptr;
  nvrtcResult (*cubin_size)(nvrtcProgram, size_t*) = nullptr;
  nvrtcResult (*cubin)(nvrtcProgram, char*) = nullptr;
  nvrtcResult (*log_size)(nvrtcProgram, size_t*) = nullptr;
  nvrtcResult (*log)(nvrtcProgram, char*) = nullptr;
  nvrtcResult (*destroy)(nvrtcProgram*) = nullptr;
};

struct Driver {
  bool ok = false;
  CUresult (*load)(CUmodule*, const void*) = nullptr;
  CUresult (*get)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream,
                     void**, void**) = nullptr;
  CUresult (*occupancy)(int*, CUfunction, int, size_t) = nullptr;
  CUresult (*set_attr)(CUfunction, CUfunction_attribute, int) = nullptr;  // optional
};

std::mutex g_mu;
Nvrtc g_nvrtc;
Driver g_drv;
bool g_loaded = false;
std::string g_why;

template <typename F>
bool sym(void* lib, const char* name, F& f) {
  f = reinterpret_cast<F>(dlsym(lib, name));
  return f != nullptr;
}

template <typename F>
bool drv_sym(const char* name, F& f) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !p) {
    cudaGetLastError();
    return false;
  }
  f = reinterpret_cast<F>(p);
  return true;
}

void load_apis() {
  if (g_loaded) return;
  g_loaded = true;
  const char* names[] = {ED_CUDA_LIB_DIR "/libnvrtc.so.13", ED_CUDA_LIB_DIR "/libnvrtc.so", "libnvrtc.so.13",
                         "libnvrtc.so"};
  void* lib = nullptr;
  for (const char* n : names)
    if ((lib = dlopen(n, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
  if (!lib) {
    g_why = "libnvrtc not found";
    return;
  }
  Nvrtc& r = g_nvrtc;
  r.ok = sym(lib, "nvrtcCreateProgram", r.create) && sym(lib, "nvrtcCompileProgram", r.compile) &&
         sym(lib, "nvrtcGetCUBINSize", r.cubin_size) && sym(lib, "nvrtcGetCUBIN", r.cubin) &&
         sym(lib, "nvrtcGetProgramLogSize", r.log_size) && sym(lib, "nvrtcGetProgramLog", r.log) &&
         sym(lib, "nvrtcDestroyProgram", r.destroy);
  Driver& d = g_drv;
  d.ok = drv_sym("cuModuleLoadData", d.load) && drv_sym("cuModuleGetFunction", d.get) &&
         drv_sym("cuLaunchKernel", d.launch) && drv_sym("cuOccupancyMaxActiveBlocksPerMultiprocessor", d.occupancy);
  if (!drv_sym("cuFuncSetAttribute", d.set_attr)) d.set_attr = nullptr;
  if (!r.ok) g_why = "NVRTC symbols missing";
  if (!d.ok) g_why = "driver entry points missing";
}

// Generated source.  The kernel names are fixed; one module per operator.
const char* kPrelude = R"(
typedef unsigned int u32;
typedef long long i64;
typedef unsigned long long u64;
struct alignas(16) D2 { double x, y; };
struct alignas(16) L2 { i64 x, y; };
#define NAN_Q ((i64)0x8000000000000000ull)
#define T0B(off) ((u32)*(const unsigned short*)((const char*)t0s + (off)))
// T0 sits in shared memory permuted by SWZ (an involution, linear over XOR):
// bits 6..10 of the index are folded into bits 1..5, which pick the bank of
// a 16-bit entry, so lanes whose indices differ only above bit 5 no longer
// meet in one bank.  T0[c ^ m] = t0s[SWZ(c) ^ SWZ(m)]: one XOR per row, and
// SWZ(m) is each bond's immediate.
#define SWZ(i) ((i) ^ ((((i) >> 6) & 31u) << 1))
// element of the fixed-point input: real parts only (RX) or (re, im) pairs
template <bool RX> struct XEt { typedef L2 T; };
template <> struct XEt<true> { typedef i64 T; };
template <bool RX> using XE = typename XEt<RX>::T;
)";

const char* kKernels = R"(
// One bond's term: the target entry when the bond flips, else zero (a select,
// not a branch, so the compiler keeps many gathers in flight).
template <bool CHECK, bool RX>
__device__ __forceinline__ void gather(const XE<RX>* p, bool on, i64& ar, i64& ai, bool& bad) {
  if (RX) {
    const i64 q = on ? *(const i64*)p : 0ll;
    if (CHECK) bad |= q == NAN_Q;
    ar += q;
  } else {
    L2 q;
    if (on) q = *(const L2*)p; else { q.x = 0; q.y = 0; }
    if (CHECK) bad |= (q.x == NAN_Q) | (q.y == NAN_Q);
    ar += q.x;
    ai += q.y;
  }
}

template <bool CHECK, bool RX, bool DOT, bool RIO>
__device__ __forceinline__ void rows(const u32* __restrict__ states, const double* __restrict__ diag,
                                     const D2* __restrict__ x, const L2* __restrict__ xq, D2* __restrict__ y,
                                     i64 dim, const unsigned short* __restrict__ t0s, const u32* __restrict__ t1, const uint4* __restrict__ t1n,
                                     double c0c, double c1c, double s1, double s2, double* dacc) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const u32 s = states[r];
    const u32 c0 = s & LOWMASK, c1 = s >> W0;
    const u32 rr = (u32)r;
    const u32 c0s = SWZ(c0);
    const u32 rb0 = rr - (u32)t0s[c0s];
    const u32 c0b = c0s << 1;  // byte offset of T0[c0]; T0[c0 ^ m] is at c0b ^ (SWZ(m) << 1)
    const u32 rb1 = rr - t1[c1];
    const uint4* __restrict__ tn = t1n + (size_t)c1 * NQ;  // t1[c1 ^ m1] of the bonds, in order
    const XE<RX>* xe = (const XE<RX>*)xq;  // rank(s) = t1[c1] + T0[c0]
    i64 a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    bool bad = false;
    BONDS
    const double d = diag[r];
    D2 xv;
    if (RIO) { xv.x = ((const double*)x)[r]; xv.y = 0.0; } else xv = x[r];
    const double s0r = (double)a0 * s1 * s2, s0i = (double)a1 * s1 * s2;
    const double s1r = (double)a2 * s1 * s2, s1i = (double)a3 * s1 * s2;
    double yr = fma(d, xv.x, fma(c0c, s0r, c1c * s1r));
    double yi = fma(d, xv.y, fma(c0c, s0i, c1c * s1i));
    if (CHECK && bad) { yr = __longlong_as_double(0x7FF8000000000000ll); yi = yr; }
    if (RIO) ((double*)y)[r] = yr;
    else { D2 o; o.x = yr; o.y = yi; y[r] = o; }
    if (DOT) {
      if (RIO) {
        dacc[0] = fma(xv.x, yr, dacc[0]);
        dacc[2] = fma(yr, yr, dacc[2]);
      } else {
        dacc[0] = fma(xv.x, yr, fma(xv.y, yi, dacc[0]));
        dacc[1] = fma(xv.x, yi, fma(-xv.y, yr, dacc[1]));
        dacc[2] = fma(yr, yr, fma(yi, yi, dacc[2]));
      }
    }
  }
}

// The checked rows (some input entry is not finite: rare) stay out of line so
// that their register needs do not weigh on the unchecked path.
template <bool RX, bool DOT, bool RIO>
__device__ __noinline__ void rows_checked(const u32* __restrict__ states, const double* __restrict__ diag,
                                          const D2* __restrict__ x, const L2* __restrict__ xq, D2* __restrict__ y,
                                          i64 dim, const unsigned short* __restrict__ t0s,
                                          const u32* __restrict__ t1, const uint4* __restrict__ t1n, double c0c, double c1c, double s1, double s2,
                                          double* dacc) {
  rows<true, RX, DOT, RIO>(states, diag, x, xq, y, dim, t0s, t1, t1n, c0c, c1c, s1, s2, dacc);
}

// RIO: x and y are real storage (double[dim]); the input is then real, and
// xq holds only real parts.  Otherwise x is complex and gmax_p[2] == 0 tells
// that it is real.
template <bool DOT, bool RIO>
__device__ __forceinline__ void body(const u32* __restrict__ states, const double* __restrict__ diag,
                                     const D2* __restrict__ x, const L2* __restrict__ xq,
                                     const int* __restrict__ gmax_p, int sbits, D2* __restrict__ y, i64 dim,
                                     const unsigned short* __restrict__ t0, const u32* __restrict__ t1, const uint4* __restrict__ t1n, double c0c,
                                     double c1c, double* __restrict__ partial) {
  extern __shared__ unsigned short t0s[];
  for (int i = threadIdx.x; i < (1 << W0); i += blockDim.x) t0s[i] = t0[SWZ((u32)i)];
  __syncthreads();
  const int e_unit = gmax_p[0] - 1022 - sbits;
  const double s1 = __longlong_as_double((i64)(e_unit / 2 + 1023) << 52);
  const double s2 = __longlong_as_double((i64)(e_unit - e_unit / 2 + 1023) << 52);
  double dacc[3] = {0.0, 0.0, 0.0};
  const bool rx = RIO || gmax_p[2] == 0;
  if (gmax_p[1]) {
    if (rx) rows_checked<true, DOT, RIO>(states, diag, x, xq, y, dim, t0s, t1, t1n, c0c, c1c, s1, s2, dacc);
    else rows_checked<false, DOT, false>(states, diag, x, xq, y, dim, t0s, t1, t1n, c0c, c1c, s1, s2, dacc);
  } else {
    if (rx) rows<false, true, DOT, RIO>(states, diag, x, xq, y, dim, t0s, t1, t1n, c0c, c1c, s1, s2, dacc);
    else if (!RIO) rows<false, false, DOT, false>(states, diag, x, xq, y, dim, t0s, t1, t1n, c0c, c1c, s1, s2, dacc);
  }
  if (DOT) {
    __shared__ double sh[3 * 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < 3; ++k) {
      double a = dacc[k];
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      if (lane == 0) sh[k * 32 + wid] = a;
    }
    __syncthreads();
    if (wid == 0) {
      for (int k = 0; k < 3; ++k) {
        double a = lane < nw ? sh[k * 32 + lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) partial[k * gridDim.x + blockIdx.x] = a;
      }
    }
  }
}

#define JIT_KERNEL(NAME, DOT, RIO, NT, MINB)                                                              \
  extern "C" __global__ void __launch_bounds__(NT, MINB) NAME(const u32* states, const double* diag,        \
      const D2* x, const L2* xq, const int* gmax_p, int sbits, D2* y, i64 dim, const unsigned short* t0,     \
      const u32* t1, const uint4* t1n, double c0c, double c1c, double* partial) {                                             \
    body<DOT, RIO>(states, diag, x, xq, gmax_p, sbits, y, dim, t0, t1, t1n, c0c, c1c, partial);                  \
  }
// register budgets: 2, 3 or 4 blocks of 256 per SM (128, 80 or 64 registers);
// _r: real storage of x and y
JIT_KERNEL(k_hv_jit_b2, false, false, 256, 2)
JIT_KERNEL(k_hv_jit_dot_b2, true, false, 256, 2)
JIT_KERNEL(k_hv_jit_b3, false, false, 256, 3)
JIT_KERNEL(k_hv_jit_dot_b3, true, false, 256, 3)
JIT_KERNEL(k_hv_jit_b4, false, false, 256, 4)
JIT_KERNEL(k_hv_jit_dot_b4, true, false, 256, 4)
JIT_KERNEL(k_hv_jit_b2_r, false, true, 256, 2)
JIT_KERNEL(k_hv_jit_dot_b2_r, true, true, 256, 2)
JIT_KERNEL(k_hv_jit_b3_r, false, true, 256, 3)
JIT_KERNEL(k_hv_jit_dot_b3_r, true, true, 256, 3)
JIT_KERNEL(k_hv_jit_b4_r, false, true, 256, 4)
JIT_KERNEL(k_hv_jit_dot_b4_r, true, true, 256, 4)
// one block per SM (one copy of T0 in shared memory, the rest of the SM's
// on-chip memory left to the L1 cache): 768 threads (80 registers) or 1024
// threads (64 registers)
JIT_KERNEL(k_hv_jit_w3, false, false, 768, 1)
JIT_KERNEL(k_hv_jit_dot_w3, true, false, 768, 1)
JIT_KERNEL(k_hv_jit_w4, false, false, 1024, 1)
JIT_KERNEL(k_hv_jit_dot_w4, true, false, 1024, 1)
JIT_KERNEL(k_hv_jit_w3_r, false, true, 768, 1)
JIT_KERNEL(k_hv_jit_dot_w3_r, true, true, 768, 1)
JIT_KERNEL(k_hv_jit_w4_r, false, true, 1024, 1)
JIT_KERNEL(k_hv_jit_dot_w4_r, true, true, 1024, 1)
)";

// Per-bond couplings: every bond has its own J_b / 2, carried as a 64-bit
// fixed-point immediate c_b; each flipped bond adds c_b * xq exactly into a
// 128-bit accumulator, and the row's sum is rounded once to FP64 (integer
// operations only), then scaled by 2^xexp.
const char* kKernelsPB = R"(
struct A128 { u64 lo; i64 hi; };
// the bonds' fixed-point couplings: a kernel parameter for the main path; the
// out-of-line checked path reads the same values from global memory
struct PBC {
  i64 c[NBC];
  __device__ __forceinline__ i64 operator[](int i) const { return c[i]; }
};
__device__ __forceinline__ void mac(A128& a, i64 q, i64 c) {
  const u64 pl = (u64)q * (u64)c;
  const i64 ph = __mul64hi(q, c);
  const u64 s = a.lo + pl;
  a.hi += ph + (i64)(s < pl);
  a.lo = s;
}

template <bool CHECK, bool RX>
__device__ __forceinline__ void gatherw(const XE<RX>* p, bool on, i64 c, A128& ar, A128& ai, bool& bad) {
  if (RX) {
    const i64 q = on ? *(const i64*)p : 0ll;
    if (CHECK) bad |= q == NAN_Q;
    mac(ar, q, c);
  } else {
    L2 q;
    if (on) q = *(const L2*)p; else { q.x = 0; q.y = 0; }
    if (CHECK) bad |= (q.x == NAN_Q) | (q.y == NAN_Q);
    mac(ar, q.x, c);
    mac(ai, q.y, c);
  }
}

// a * 2^X rounded to nearest even (integer operations; below 2^-1022 -> 0)
__device__ __forceinline__ double a128_to_double(A128 a, int X) {
  u64 lo = a.lo;
  i64 hi = a.hi;
  const bool neg = hi < 0;
  if (neg) { lo = ~lo + 1ull; hi = ~hi + (lo == 0ull ? 1ll : 0ll); }
  const u64 uh = (u64)hi;
  if (uh == 0ull && lo == 0ull) return 0.0;
  const int L = uh ? 128 - __clzll((i64)uh) : 64 - __clzll((i64)lo);
  u64 m;
  int bexp = X + L + 1022;
  if (L <= 53) {
    m = lo << (53 - L);
  } else {
    const int sr = L - 53;  // 1 .. 75
    u64 top, rest;
    if (sr < 64) { top = (lo >> sr) | (uh << (64 - sr)); rest = lo & ((1ull << sr) - 1ull); }
    else { top = uh >> (sr - 64); rest = (sr > 64 ? (uh & ((1ull << (sr - 64)) - 1ull)) : 0ull) | lo; }
    m = top;
    const u64 half = sr < 64 ? (1ull << (sr - 1)) : 0ull;
    bool up;
    if (sr < 64) up = rest > half || (rest == half && (m & 1ull));
    else {
      const u64 hb = sr == 64 ? (lo >> 63) : ((uh >> (sr - 65)) & 1ull);
      const u64 below = sr == 64 ? (lo << 1) : ((uh & ((1ull << (sr - 65)) - 1ull)) | lo);
      up = hb && (below != 0ull || (m & 1ull));
    }
    m += up ? 1ull : 0ull;
    if (m >> 53) { m >>= 1; ++bexp; }
  }
  if (bexp <= 0) return 0.0;
  return __longlong_as_double((i64)(((u64)neg << 63) | ((u64)bexp << 52) | (m & 0xFFFFFFFFFFFFFull)));
}

template <bool CHECK, bool RX, bool DOT, bool RIO, typename CF>
__device__ __forceinline__ void rows(const u32* __restrict__ states, const double* __restrict__ diag,
                                     const D2* __restrict__ x, const L2* __restrict__ xq, D2* __restrict__ y,
                                     i64 dim, const unsigned short* __restrict__ t0s, const u32* __restrict__ t1, const uint4* __restrict__ t1n,
                                     int xexp, double* dacc, const CF& cf) {
  const i64 stride = (i64)gridDim.x * blockDim.x;
  for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += stride) {
    const u32 s = states[r];
    const u32 c0 = s & LOWMASK, c1 = s >> W0;
    const u32 rr = (u32)r;
    const u32 c0s = SWZ(c0);
    const u32 rb0 = rr - (u32)t0s[c0s];
    const u32 c0b = c0s << 1;
    const u32 rb1 = rr - t1[c1];
    const uint4* __restrict__ tn = t1n + (size_t)c1 * NQ;  // t1[c1 ^ m1] of the bonds, in order
    const XE<RX>* xe = (const XE<RX>*)xq;  // rank(s) = t1[c1] + T0[c0]
    A128 ar = {0ull, 0ll}, ai = {0ull, 0ll};
    bool bad = false;
    BONDS
    const double d = diag[r];
    D2 xv;
    if (RIO) { xv.x = ((const double*)x)[r]; xv.y = 0.0; } else xv = x[r];
    double yr = fma(d, xv.x, a128_to_double(ar, xexp));
    double yi = RX ? d * xv.y : fma(d, xv.y, a128_to_double(ai, xexp));
    if (CHECK && bad) { yr = __longlong_as_double(0x7FF8000000000000ll); yi = yr; }
    if (RIO) ((double*)y)[r] = yr;
    else { D2 o; o.x = yr; o.y = yi; y[r] = o; }
    if (DOT) {
      if (RIO) {
        dacc[0] = fma(xv.x, yr, dacc[0]);
        dacc[2] = fma(yr, yr, dacc[2]);
      } else {
        dacc[0] = fma(xv.x, yr, fma(xv.y, yi, dacc[0]));
        dacc[1] = fma(xv.x, yi, fma(-xv.y, yr, dacc[1]));
        dacc[2] = fma(yr, yr, fma(yi, yi, dacc[2]));
      }
    }
  }
}

template <bool RX, bool DOT, bool RIO>
__device__ __noinline__ void rows_checked(const u32* __restrict__ states, const double* __restrict__ diag,
                                          const D2* __restrict__ x, const L2* __restrict__ xq, D2* __restrict__ y,
                                          i64 dim, const unsigned short* __restrict__ t0s,
                                          const u32* __restrict__ t1, const uint4* __restrict__ t1n, int xexp, double* dacc,
                                          const i64* __restrict__ gcf) {
  rows<true, RX, DOT, RIO>(states, diag, x, xq, y, dim, t0s, t1, t1n, xexp, dacc, gcf);
}

template <bool DOT, bool RIO>
__device__ __forceinline__ void body(const u32* __restrict__ states, const double* __restrict__ diag,
                                     const D2* __restrict__ x, const L2* __restrict__ xq,
                                     const int* __restrict__ gmax_p, int sbits, D2* __restrict__ y, i64 dim,
                                     const unsigned short* __restrict__ t0, const u32* __restrict__ t1, const uint4* __restrict__ t1n, int pbexp,
                                     double* __restrict__ partial, const PBC& pbc, const i64* __restrict__ gcf) {
  extern __shared__ unsigned short t0s[];
  for (int i = threadIdx.x; i < (1 << W0); i += blockDim.x) t0s[i] = t0[SWZ((u32)i)];
  __syncthreads();
  const int xexp = gmax_p[0] - 1022 - sbits + pbexp;
  double dacc[3] = {0.0, 0.0, 0.0};
  const bool rx = RIO || gmax_p[2] == 0;
  if (gmax_p[1]) {
    if (rx) rows_checked<true, DOT, RIO>(states, diag, x, xq, y, dim, t0s, t1, t1n, xexp, dacc, gcf);
    else rows_checked<false, DOT, false>(states, diag, x, xq, y, dim, t0s, t1, t1n, xexp, dacc, gcf);
  } else {
    if (rx) rows<false, true, DOT, RIO>(states, diag, x, xq, y, dim, t0s, t1, t1n, xexp, dacc, pbc);
    else if (!RIO) rows<false, false, DOT, false>(states, diag, x, xq, y, dim, t0s, t1, t1n, xexp, dacc, pbc);
  }
  if (DOT) {
    __shared__ double sh[3 * 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < 3; ++k) {
      double a = dacc[k];
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      if (lane == 0) sh[k * 32 + wid] = a;
    }
    __syncthreads();
    if (wid == 0) {
      for (int k = 0; k < 3; ++k) {
        double a = lane < nw ? sh[k * 32 + lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) partial[k * gridDim.x + blockIdx.x] = a;
      }
    }
  }
}

#define JIT_KERNEL(NAME, DOT, RIO, NT, MINB)                                                              \
  extern "C" __global__ void __launch_bounds__(NT, MINB) NAME(const u32* states, const double* diag,        \
      const D2* x, const L2* xq, const int* gmax_p, int sbits, D2* y, i64 dim, const unsigned short* t0,     \
      const u32* t1, const uint4* t1n, int pbexp, double* partial, const __grid_constant__ PBC pbc, const i64* gcf) {         \
    body<DOT, RIO>(states, diag, x, xq, gmax_p, sbits, y, dim, t0, t1, t1n, pbexp, partial, pbc, gcf);           \
  }
JIT_KERNEL(k_hv_jit_b2, false, false, 256, 2)
JIT_KERNEL(k_hv_jit_dot_b2, true, false, 256, 2)
JIT_KERNEL(k_hv_jit_b3, false, false, 256, 3)
JIT_KERNEL(k_hv_jit_dot_b3, true, false, 256, 3)
JIT_KERNEL(k_hv_jit_b4, false, false, 256, 4)
JIT_KERNEL(k_hv_jit_dot_b4, true, false, 256, 4)
JIT_KERNEL(k_hv_jit_b2_r, false, true, 256, 2)
JIT_KERNEL(k_hv_jit_dot_b2_r, true, true, 256, 2)
JIT_KERNEL(k_hv_jit_b3_r, false, true, 256, 3)
JIT_KERNEL(k_hv_jit_dot_b3_r, true, true, 256, 3)
JIT_KERNEL(k_hv_jit_b4_r, false, true, 256, 4)
JIT_KERNEL(k_hv_jit_dot_b4_r, true, true, 256, 4)
// one block per SM (one copy of T0 in shared memory, the rest of the SM's
// on-chip memory left to the L1 cache): 768 threads (80 registers) or 1024
// threads (64 registers)
JIT_KERNEL(k_hv_jit_w3, false, false, 768, 1)
JIT_KERNEL(k_hv_jit_dot_w3, true, false, 768, 1)
JIT_KERNEL(k_hv_jit_w4, false, false, 1024, 1)
JIT_KERNEL(k_hv_jit_dot_w4, true, false, 1024, 1)
JIT_KERNEL(k_hv_jit_w3_r, false, true, 768, 1)
JIT_KERNEL(k_hv_jit_dot_w3_r, true, true, 768, 1)
JIT_KERNEL(k_hv_jit_w4_r, false, true, 1024, 1)
JIT_KERNEL(k_hv_jit_dot_w4_r, true, true, 1024, 1)
)";

// Register budgets of the generated kernels, by the budget index of
// ed_jit_launch: 0, 1, 2 = two, four, three blocks of 256 per SM; 3, 4 = one
// block of 768 or 1024 per SM.
const int kJitBudgets = 5;
const char* const kJitBudgetSuffix[kJitBudgets] = {"b2", "b4", "b3", "w3", "w4"};
const int kJitThreads[kJitBudgets] = {256, 256, 256, 768, 1024};

struct JitModule {
  bool ok = false;
  CUfunction fn[kJitBudgets][2][2] = {};  // [budget][dot][real storage]
  int per_sm[kJitBudgets][2][2] = {};
  std::vector<uint32_t> slots;  // high-half mask of each neighbour-table slot
  int nq = 1;                   // 16-byte loads per row of the neighbour table
};

std::map<std::tuple<int, uint64_t>, JitModule> g_modules;

// On-disk cache of compiled modules (the compile takes seconds): directory
// $ED_JIT_CACHE, else $XDG_CACHE_HOME/lsquantumed_gb300, else
// $HOME/.cache/lsquantumed_gb300; file name = hash of the source and options.
std::string cache_dir() {
  if (const char* d = getenv("ED_JIT_CACHE")) return d;
  if (const char* d = getenv("XDG_CACHE_HOME")) return std::string(d) + "/lsquantumed_gb300";
  if (const char* d = getenv("HOME")) return std::string(d) + "/.cache/lsquantumed_gb300";
  return "";
}

uint64_t fnv(const std::string& s) {
  uint64_t z = 1469598103934665603ull;
  for (unsigned char c : s) { z ^= c; z *= 1099511628211ull; }
  return z;
}

bool cache_read(const std::string& path, std::vector<char>& out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  out.resize(n > 0 ? (size_t)n : 0);
  const bool ok = n > 0 && fread(out.data(), 1, (size_t)n, f) == (size_t)n;
  fclose(f);
  return ok;
}

void cache_write(const std::string& dir, const std::string& path, const std::vector<char>& data) {
  if (dir.empty()) return;
  std::string cur;
  for (size_t i = 0; i <= dir.size(); ++i) {  // mkdir -p
    if (i == dir.size() || dir[i] == '/') {
      if (!cur.empty()) mkdir(cur.c_str(), 0755);
    }
    if (i < dir.size()) cur += dir[i];
  }
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return;
  const bool ok = fwrite(data.data(), 1, data.size(), f) == data.size();
  fclose(f);
  if (ok) rename(tmp.c_str(), path.c_str());
  else remove(tmp.c_str());
}

std::string hex(uint32_t v) {
  char b[16];
  snprintf(b, sizeof(b), "0x%xu", v);
  return b;
}

// Flip test of a bond: with the bond's sites lo < hi in the state word, the
// spins differ when bit lo of z_d = s ^ (s >> d), d = hi - lo, is set: one
// AND with an immediate per bond.  The bonds are emitted grouped by d, each
// group after its z_d, so that one z_d is live at a time.  A mask that is not
// two distinct sites never flips (d = -1).
std::string flip_test(uint32_t m0, uint32_t m1, int w0, int* d_out) {
  const uint64_t m = (uint64_t)m0 | ((uint64_t)m1 << w0);
  *d_out = -1;
  if (__builtin_popcountll(m) != 2) return "false";
  const int lo = __builtin_ctzll(m), hi = 63 - __builtin_clzll(m);
  *d_out = hi - lo;
  return "((z" + std::to_string(hi - lo) + " & " + hex(1u << lo) + ") != 0u)";
}

// Address of a bond's target entry, rank(s ^ m): class 0 (both sites in the
// low half), 1 (both in the high half), 2 (across).
// the shared-memory T0's permutation (SWZ in the generated source)
uint32_t swz(uint32_t i) { return i ^ (((i >> 6) & 31u) << 1); }

// t1v: the expression of t1[c1 ^ m1] (a component of a 16-byte load from
// the row's neighbour table)
std::string target(int cls, uint32_t m0, const std::string& t1v) {
  if (cls == 0) return "xe + (rb0 + T0B(c0b ^ " + hex(swz(m0) << 1) + "))";
  if (cls == 1) return "xe + (rb1 + " + t1v + ")";
  return "xe + (T0B(c0b ^ " + hex(swz(m0) << 1) + ") + " + t1v + ")";
}

// One bond's code; type selects the accumulators (nn: a0/a1, nnn: a2/a3).
std::string bond_code(int cls, int type, uint32_t m0, uint32_t m1, const std::string& t1v, int w0, int* d) {
  const char* ar = type ? "a2" : "a0";
  const char* ai = type ? "a3" : "a1";
  const std::string on = flip_test(m0, m1, w0, d);
  return "gather<CHECK, RX>(" + target(cls, m0, t1v) + ", " + on + ", " + ar + ", " + ai + ", bad);\n    ";
}

// Per-bond form: the bond's own coefficient (entry q of the kernel's
// coefficient parameter) instead of a type accumulator.
std::string bond_code_pb(int cls, uint32_t m0, uint32_t m1, const std::string& t1v, int q, int w0, int* d) {
  const std::string on = flip_test(m0, m1, w0, d);
  return "gatherw<CHECK, RX>(" + target(cls, m0, t1v) + ", " + on + ", cf[" + std::to_string(q) + "], ar, ai, bad);\n    ";
}

// out[c1][k] = t1[c1 ^ slots[k]] (0 past the last slot), nq * 4 entries per c1
__global__ void k_build_t1n(const uint32_t* __restrict__ t1, int64_t nc1, const uint32_t* __restrict__ slots, int K,
                            int nq, uint32_t* __restrict__ out) {
  const int64_t per = (int64_t)nq * 4, n = nc1 * per;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t c1 = i / per;
    const int k = (int)(i - c1 * per);
    out[i] = k < K ? t1[(uint32_t)c1 ^ slots[k]] : 0u;
  }
}

}  // namespace

bool ed_jit_available() {
  std::lock_guard<std::mutex> lk(g_mu);
  load_apis();
  return g_nvrtc.ok && g_drv.ok;
}

// Signature of the operator's bond words (the same hash the autotuner keys on).
int ed_jit_launch(ed_ham* h, uint64_t signature, int budget, const void* x, void* y, bool dot, int sbits,
                  int* nblk_out, const unsigned long long* words, const int* seg, int w0, bool rio,
                  const long long* coef, const long long* coef_dev, int pbexp) {
  ed_ctx* ctx = h->ctx;
  const ed_basis* b = h->basis;
  JitModule* mod = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    load_apis();
    if (!g_nvrtc.ok || !g_drv.ok) return ed_fail(ED_ENOTSUP, "run-time compilation unavailable: " + g_why);
    auto key = std::make_tuple(ctx->device, signature);
    auto it = g_modules.find(key);
    if (it == g_modules.end()) {
      JitModule jm;
      // the bonds grouped by d, each group after its z_d; t1[c1 ^ m1] of the
      // high-half and crossing bonds come from the row's neighbour table, in
      // slots numbered in emission order (crossing bonds of one m1 share a
      // slot), four per 16-byte load, each load emitted before its first use
      struct Bond { int cls, t, q, d; uint32_t m0, m1; };
      std::vector<Bond> bonds;
      std::vector<int> dists;
      for (int cls = 0; cls < 3; ++cls)
        for (int t = 0; t < 2; ++t)
          for (int q = seg[cls * 2 + t]; q < seg[cls * 2 + t + 1]; ++q) {
            Bond bd{cls, t, q, -1, (uint32_t)words[q], (uint32_t)(words[q] >> 32)};
            flip_test(bd.m0, bd.m1, w0, &bd.d);
            if (bd.d < 0) continue;  // never flips
            if (std::find(dists.begin(), dists.end(), bd.d) == dists.end()) dists.push_back(bd.d);
            bonds.push_back(bd);
          }
      std::vector<uint32_t> slot_m1;
      std::map<uint32_t, int> cross_slot;
      std::ostringstream body;
      std::ostringstream decl;
      for (int d : dists) {
        body << "{ const u32 z" << d << " = s ^ (s >> " << d << "u);\n    ";
        for (const Bond& bd : bonds) {
          if (bd.d != d) continue;
          std::string t1v;
          if (bd.cls != 0) {
            int k;
            auto it = bd.cls == 2 ? cross_slot.find(bd.m1) : cross_slot.end();
            if (it != cross_slot.end()) {
              k = it->second;
            } else {
              k = (int)slot_m1.size();
              slot_m1.push_back(bd.m1);
              if (bd.cls == 2) cross_slot[bd.m1] = k;
              if (k % 4 == 0) body << "Q" << k / 4 << " = tn[" << k / 4 << "];\n    ";
            }
            static const char* comp[4] = {".x", ".y", ".z", ".w"};
            t1v = "Q" + std::to_string(k / 4) + comp[k % 4];
          }
          int dd = -1;
          body << (coef ? bond_code_pb(bd.cls, bd.m0, bd.m1, t1v, bd.q, w0, &dd)
                        : bond_code(bd.cls, bd.t, bd.m0, bd.m1, t1v, w0, &dd));
        }
        body << "}\n    ";
      }
      const int nq = std::max(1, ((int)slot_m1.size() + 3) / 4);
      for (int k = 0; k < (int)(slot_m1.size() + 3) / 4; ++k) decl << "uint4 Q" << k << ";\n    ";
      jm.slots = slot_m1;
      jm.nq = nq;
      std::string kern = coef ? kKernelsPB : kKernels;
      const size_t at = kern.find("BONDS");
      kern.replace(at, 5, decl.str() + body.str());
      std::string src = std::string(kPrelude) + "#define W0 " + std::to_string(w0) + "\n#define LOWMASK " +
                        hex((1u << w0) - 1u) + "\n#define NBC " + std::to_string(std::max(1, seg[6])) +
                        "\n#define NQ " + std::to_string(nq) + "\n" + kern;
      const char* opts[] = {"-arch=sm_103a", "-std=c++17", "-default-device"};
      const std::string dir = cache_dir();
      char name[40];
      snprintf(name, sizeof(name), "/hv_%016llx.cubin",
               (unsigned long long)fnv(src + opts[0] + opts[1] + opts[2]));
      const std::string path = dir.empty() ? std::string() : dir + name;
      std::vector<char> cubin;
      if (path.empty() || !cache_read(path, cubin)) {
        nvrtcProgram prog;
        if (g_nvrtc.create(&prog, src.c_str(), "ed_hv_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
          return ed_fail(ED_ENOTSUP, "nvrtcCreateProgram failed");
        nvrtcResult cr = g_nvrtc.compile(prog, 3, opts);
        if (cr != NVRTC_SUCCESS) {
          size_t n = 0;
          g_nvrtc.log_size(prog, &n);
          std::string log(n, '\0');
          if (n) g_nvrtc.log(prog, &log[0]);
          g_nvrtc.destroy(&prog);
          g_modules[key] = jm;  // remember the failure: do not retry every call
          return ed_fail(ED_ENOTSUP, "run-time compilation failed: " + log.substr(0, 400));
        }
        size_t n = 0;
        g_nvrtc.cubin_size(prog, &n);
        cubin.resize(n);
        g_nvrtc.cubin(prog, cubin.data());
        g_nvrtc.destroy(&prog);
        cache_write(dir, path, cubin);
      }
      CUmodule m = nullptr;
      bool got = g_drv.load(&m, cubin.data()) == CUDA_SUCCESS;
      const size_t smem = sizeof(uint16_t) * ((size_t)1 << w0);
      for (int bg = 0; bg < kJitBudgets && got; ++bg)
        for (int k = 0; k < 2 && got; ++k)
          for (int ri = 0; ri < 2 && got; ++ri) {
            const std::string fname = std::string(k ? "k_hv_jit_dot_" : "k_hv_jit_") + kJitBudgetSuffix[bg] +
                                      (ri ? "_r" : "");
            got = g_drv.get(&jm.fn[bg][k][ri], m, fname.c_str()) == CUDA_SUCCESS;
            if (got && kJitThreads[bg] > 256) {
              // a single block per SM needs only its copy of T0: ask for the
              // smallest shared-memory carveout that holds it (a hint)
              const int pct = (int)std::min<size_t>(100, ((smem + 1024) * 100 + 228 * 1024 - 1) / (228 * 1024));
              if (g_drv.set_attr) g_drv.set_attr(jm.fn[bg][k][ri], CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, pct);
            }
            int ps = 0;
            if (got && (g_drv.occupancy(&ps, jm.fn[bg][k][ri], kJitThreads[bg], smem) != CUDA_SUCCESS || ps < 1))
              ps = 1;
            jm.per_sm[bg][k][ri] = ps;
          }
      if (!got) {
        g_modules[key] = jm;
        return ed_fail(ED_ENOTSUP, "loading the compiled H.v module failed");
      }
      jm.ok = true;
      it = g_modules.emplace(key, jm).first;
    }
    if (!it->second.ok) return ed_fail(ED_ENOTSUP, "run-time compiled H.v unavailable for this operator");
    mod = &it->second;
  }
  const size_t smem = sizeof(uint16_t) * ((size_t)1 << w0);
  if (budget < 0 || budget >= kJitBudgets) return ed_fail(ED_EINVAL, "unknown register budget");
  if (h->jit_t1n_key != (const void*)mod) {
    // this operator's neighbour table for the module's slot order
    const int K = (int)mod->slots.size();
    const int64_t nc1 = (int64_t)1 << (b->nspins - w0);
    const size_t bytes = sizeof(uint32_t) * ((size_t)nc1 * mod->nq * 4 + (size_t)std::max(K, 1));
    if (h->jit_t1n) cudaFree(h->jit_t1n);
    h->jit_t1n = nullptr;
    h->jit_t1n_key = nullptr;
    if (cudaMalloc(&h->jit_t1n, bytes) != cudaSuccess) {
      cudaGetLastError();
      h->jit_t1n = nullptr;
      return ed_fail(ED_ENOMEM, "neighbour table of the run-time compiled H.v does not fit in device memory");
    }
    uint32_t* tab = (uint32_t*)h->jit_t1n;
    uint32_t* dslots = tab + (size_t)nc1 * mod->nq * 4;
    if (K > 0)
      ED_CUDA(cudaMemcpyAsync(dslots, mod->slots.data(), sizeof(uint32_t) * K, cudaMemcpyHostToDevice, ctx->stream));
    const int gb = (int)std::max<int64_t>(1, std::min<int64_t>(nc1 * mod->nq * 4 / 256 + 1, (int64_t)ctx->num_sms * 8));
    k_build_t1n<<<gb, 256, 0, ctx->stream>>>(b->d_lin_t1, nc1, dslots, K, mod->nq, tab);
    ED_CHECK_LAUNCH(ctx);
    ED_CUDA(cudaStreamSynchronize(ctx->stream));  // the slot list is pageable host memory
    h->jit_t1n_key = (const void*)mod;
  }
  const int bg = budget, kd = dot ? 1 : 0, ri = rio ? 1 : 0;
  const int nt = kJitThreads[bg];
  int64_t g = (b->dim + nt - 1) / nt;
  g = std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx->num_sms * mod->per_sm[bg][kd][ri]));
  const int nblk = (int)g;
  if (dot) ED_TRY(ed_ensure_reduce(ctx, (size_t)3 * nblk + 8));
  const uint32_t* states = b->d_states;
  const double* diag = h->d_diag;
  const longlong2* xq = h->d_xq;
  const int* gmax = h->d_gmax;
  int64_t dim = b->dim;
  const uint16_t* t0 = b->d_lin_t0;
  const uint32_t* t1 = b->d_lin_t1;
  double c0c = h->bs.chalf[0], c1c = h->bs.chalf[1];
  double* partial = dot ? ctx->d_red : nullptr;
  const void* t1n = h->jit_t1n;
  void* args_u[] = {&states, &diag, &x, &xq, &gmax, &sbits, &y, &dim, &t0, &t1, &t1n, &c0c, &c1c, &partial};
  std::vector<long long> pbc(coef ? std::max(1, seg[6]) : 0, 0ll);  // the PBC parameter's bytes
  if (coef) std::copy(coef, coef + seg[6], pbc.begin());
  void* args_pb[] = {&states, &diag, &x, &xq, &gmax, &sbits, &y, &dim, &t0, &t1, &t1n, &pbexp, &partial, pbc.data(),
                     &coef_dev};
  void** args = coef ? args_pb : args_u;
  CUresult r = g_drv.launch(mod->fn[bg][kd][ri], (unsigned)nblk, 1, 1, (unsigned)nt, 1, 1, (unsigned)smem,
                            (CUstream)ctx->stream, args, nullptr);
  if (r != CUDA_SUCCESS) return ed_fail(ED_ECUDA, "launch of the compiled H.v failed");
  ctx->kernels++;
  if (nblk_out) *nblk_out = nblk;
  return ED_OK;
}
