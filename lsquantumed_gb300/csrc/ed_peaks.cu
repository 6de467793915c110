// Arithmetic-rate probes behind the choice of units for the dense
// contractions of the eigensolve (Gram-Schmidt dots and update, restart
// combination): FP64 FMA on the vector pipe, FP64 on the tensor pipe
// (mma.sync m8n8k4 f64), and the FP16-input / FP32-accumulate tensor path
// that the exact-slice kernels use (mma.sync m16n8k16, the warp-level form).
// Each probe runs a register-resident loop with independent accumulators on
// every SM, timed with CUDA events; the results are throughputs in TFLOP/s
// (two flops per multiply-add).  No counterpart in the reference.
#include "ed_internal.h"
#include <cuda_fp16.h>

namespace {

constexpr int PK_ITERS = 4096;
constexpr int PK_THREADS = 256;

__global__ void __launch_bounds__(PK_THREADS) k_peak_dfma(double seed, double* sink) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-9 + k;
  const double b = 1.0 - 1e-12, c = 1e-13;
  for (int it = 0; it < PK_ITERS; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 12345.678) sink[0] = s;  // never true; keeps the loop
}

__global__ void __launch_bounds__(PK_THREADS) k_peak_dmma(double seed, double* sink) {
  // per warp: 4 independent 8x8 accumulators, D = A(8x4) B(4x8) + D
  double acc[4][2];
#pragma unroll
  for (int k = 0; k < 4; ++k) acc[k][0] = acc[k][1] = seed * k;
  const double a = 1.0 + threadIdx.x * 1e-12, b = 1.0 - 1e-12;
  for (int it = 0; it < PK_ITERS; ++it) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(acc[k][0]), "+d"(acc[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) s += acc[k][0] + acc[k][1];
  if (s == 12345.678) sink[0] = s;
}

__global__ void __launch_bounds__(PK_THREADS) k_peak_hmma(float seed, float* sink) {
  // per warp: 4 independent 16x8 FP32 accumulators, D = A(16x16) B(16x8) + D, FP16 inputs
  float acc[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[k][q] = seed * k;
  const __half2 h = __floats2half2_rn(1.0f, 0.5f);
  const unsigned hv = *reinterpret_cast<const unsigned*>(&h);
  for (int it = 0; it < PK_ITERS; ++it) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                   "{%8, %9}, {%0, %1, %2, %3};"
                   : "+f"(acc[k][0]), "+f"(acc[k][1]), "+f"(acc[k][2]), "+f"(acc[k][3])
                   : "r"(hv), "r"(hv), "r"(hv), "r"(hv), "r"(hv), "r"(hv));
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) s += acc[k][0] + acc[k][1] + acc[k][2] + acc[k][3];
  if (s == 12345.678f) sink[0] = s;
}

template <typename F>
int time_probe(ed_ctx* ctx, F launch, double flops, double* tflops) {
  cudaEvent_t e0, e1;
  ED_CUDA(cudaEventCreate(&e0));
  ED_CUDA(cudaEventCreate(&e1));
  launch();  // warm-up
  ED_CHECK_LAUNCH(ctx);
  ED_CUDA(cudaEventRecord(e0, ctx->stream));
  const int reps = 5;
  for (int r = 0; r < reps; ++r) {
    launch();
    ED_CHECK_LAUNCH(ctx);
  }
  ED_CUDA(cudaEventRecord(e1, ctx->stream));
  ED_CUDA(cudaEventSynchronize(e1));
  float ms = 0.0f;
  ED_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tflops = flops * reps / (ms * 1e-3) / 1e12;
  return ED_OK;
}

}  // namespace

extern "C" int ed_probe_rates(ed_ctx* ctx, double* dfma_tflops, double* dmma_tflops, double* hmma_tflops) {
  if (!ctx) return ed_fail(ED_EINVAL, "null context");
  double* sink = nullptr;
  ED_CUDA(cudaMalloc(&sink, 64));
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_peak_dfma, PK_THREADS, 0);
  const int grid = ctx->num_sms * std::max(per_sm, 1);
  const double threads = (double)grid * PK_THREADS;
  int rc = ED_OK;
  if (dfma_tflops)
    rc = time_probe(ctx, [&] { k_peak_dfma<<<grid, PK_THREADS, 0, ctx->stream>>>(1.0, sink); },
                    threads * PK_ITERS * 8 * 2.0, dfma_tflops);
  // per warp and mma: 8x8x4 multiply-adds (f64), 16x8x16 (f16)
  const double warps = threads / 32.0;
  if (rc == ED_OK && dmma_tflops)
    rc = time_probe(ctx, [&] { k_peak_dmma<<<grid, PK_THREADS, 0, ctx->stream>>>(1.0, sink); },
                    warps * PK_ITERS * 4 * (8.0 * 8 * 4 * 2), dmma_tflops);
  if (rc == ED_OK && hmma_tflops)
    rc = time_probe(ctx, [&] { k_peak_hmma<<<grid, PK_THREADS, 0, ctx->stream>>>(1.0f, (float*)sink); },
                    warps * PK_ITERS * 4 * (16.0 * 8 * 16 * 2), hmma_tflops);
  cudaFree(sink);
  return rc;
}
