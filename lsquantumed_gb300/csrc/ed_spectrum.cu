// Dynamical structure factor S(q, w) from the DSF coefficients, on the device.
//
// Restates the post-processing of postprocessing/dynamicStep0_preprocess.ipynb:
//   cell 12-13: F[q][n] = |sum_i e^{i q.r_i} c[i][n]|^2 / N
//   cell 11:    delta(w, dE) = (1/pi) eps^2 / (eps^2 + (w - dE)^2)
//   cell 15:    S[q][k] = sum_n F[q][n] delta(w_k, dE[n]),  w_k = linspace(w_min, w_max, nw)
//   cell 17:    the disorder average 2 pi / rep * sum over realisations (done by
//               accumulating realisations into S and scaling once).
// One thread per (q, n) for F, one thread per (q, k) for S (sum over n in
// level order, as the notebook's np.sum over the level axis).
#include "ed_internal.h"
#include <algorithm>
#include <cmath>
#include <vector>

__global__ void k_dsf_factor(int nspins, int nev, const double2* __restrict__ c, int nq, const double* __restrict__ q,
                             const double* __restrict__ r, double* __restrict__ F) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq * nev) return;
  const int iq = t / nev, n = t % nev;
  double ar = 0.0, ai = 0.0;
  for (int i = 0; i < nspins; ++i) {
    const double ph = q[2 * iq] * r[2 * i] + q[2 * iq + 1] * r[2 * i + 1];
    double s, co;
    sincos(ph, &s, &co);
    const double2 cc = c[(size_t)i * nev + n];
    ar += co * cc.x - s * cc.y;
    ai += co * cc.y + s * cc.x;
  }
  F[t] = (ar * ar + ai * ai) / nspins;
}

__global__ void k_dsf_lorentz(int nev, const double* __restrict__ F, const double* __restrict__ dE, int nq, int nw,
                              double w_min, double dw, double eps, double* __restrict__ S) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nq * nw) return;
  const int iq = (int)(t / nw), k = (int)(t % nw);
  const double w = w_min + k * dw;
  const double e2 = eps * eps, inv_pi = 1.0 / 3.141592653589793;
  double acc = 0.0;
  for (int n = 0; n < nev; ++n) {
    const double d = w - dE[n];
    acc += F[(size_t)iq * nev + n] * (inv_pi * e2 / (e2 + d * d));
  }
  S[t] += acc;
}

extern "C" int ed_dsf_spectrum(ed_ctx* ctx, int nspins, int nev, const ed_cplx* c_host, const double* dE_host, int nq,
                               const double* q_host, const double* r_host, int nw, double w_min, double w_max,
                               double eps, double* S_dev) {
  if (!ctx || !c_host || !dE_host || !q_host || !r_host || !S_dev) return ed_fail(ED_EINVAL, "null argument");
  if (nspins < 1 || nev < 1 || nq < 1 || nw < 2) return ed_fail(ED_EINVAL, "nspins, nev, nq >= 1 and nw >= 2");
  if (!(eps > 0.0)) return ed_fail(ED_EINVAL, "eps must be positive");
  const size_t nc = (size_t)nspins * nev;
  const size_t bytes = sizeof(double2) * nc + sizeof(double) * ((size_t)nev + 2 * (size_t)nq + 2 * (size_t)nspins +
                                                                (size_t)nq * nev);
  char* buf = nullptr;
  ED_CUDA(cudaMalloc(&buf, bytes));
  double2* c = (double2*)buf;
  double* dE = (double*)(c + nc);
  double* q = dE + nev;
  double* r = q + 2 * (size_t)nq;
  double* F = r + 2 * (size_t)nspins;
  cudaError_t e = cudaMemcpyAsync(c, c_host, sizeof(double2) * nc, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dE, dE_host, sizeof(double) * nev, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(q, q_host, sizeof(double) * 2 * nq, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(r, r_host, sizeof(double) * 2 * nspins, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    const int nt = nq * nev;
    k_dsf_factor<<<(nt + 127) / 128, 128, 0, ctx->stream>>>(nspins, nev, c, nq, q, r, F);
    e = cudaGetLastError();
    if (e == cudaSuccess) ctx->kernels++;
  }
  if (e == cudaSuccess) {
    const int64_t nt = (int64_t)nq * nw;
    const double dw = (w_max - w_min) / (nw - 1);
    k_dsf_lorentz<<<(unsigned)((nt + 255) / 256), 256, 0, ctx->stream>>>(nev, F, dE, nq, nw, w_min, dw, eps, S_dev);
    e = cudaGetLastError();
    if (e == cudaSuccess) ctx->kernels++;
  }
  // the host inputs must stay valid until the copies ran
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(buf);
  if (e != cudaSuccess) return ed_cuda_fail(e, "DSF spectrum", __FILE__, __LINE__);
  return ED_OK;
}
