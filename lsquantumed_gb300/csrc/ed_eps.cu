// Krylov-Schur eigensolver for the Hermitian Hamiltonian (lowest eigenvalues),
// replacing Solver::SolverInit / solve / solution / SolverClean
// (src/solver.cpp:7-68), i.e. SLEPc EPS with EPS_HEP, EPSKRYLOVSCHUR and
// EPS_SMALLEST_REAL.
//
// Method (Stewart's Krylov-Schur, thick-restart Lanczos form for Hermitian
// operators): expand the basis to ncv vectors with H.v and classical
// Gram-Schmidt plus one conditional refinement (eta = 1/sqrt(2), SLEPc's
// default "refine if needed" criterion); solve the small real-symmetric
// arrowhead+tridiagonal projected problem on the host in FP64; count leading
// Ritz pairs whose residual estimate |beta_m y_{m,i}| / |theta_i| is below
// tol (EPS_CONV_REL); keep nconv + max(1, (m - nconv)/2) Ritz vectors and
// restart.  Vectors stay on the device; only the small projected matrix and
// the Gram-Schmidt coefficients cross to the host.
#include "ed_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

struct ed_eps {
  ed_ham* h = nullptr;
  int nev = 1, ncv = 0, mpd = 0;
  double tol = 0.0;
  int max_it = 0;
  uint64_t seed = 0;
  bool solved = false;
  int nconv = 0, its = 0, nrep = 0;
  int64_t nhv = 0;
  int64_t ortho_passes = 0;
  bool real_coeffs = true;            // see orthogonalize_lanczos
  std::vector<double> evals, errs;
  double2* pool = nullptr;            // column storage
  int pool_cols = 0;
  double2* w = nullptr;
  std::vector<double2*> col;          // current basis columns (after solve: Ritz vectors)
  double2* v0 = nullptr;              // user initial vector (EPSSetInitialSpace)
  // real storage (real mode with the two-table H.v): columns hold only the
  // real parts of the basis, whose imaginary parts are exactly zero
  bool real_storage = false;
  double* pool_r = nullptr;
  double* w_r = nullptr;
  std::vector<double*> col_r;
  int restart_arith = ED_RESTART_AUTO;  // ed_eps_set_restart_arithmetic
  int restart_mode = ED_RESTART_FP64;   // the form this real-storage solve uses
};

void ed_jacobi_eig(int m, std::vector<double>& A, std::vector<double>& theta, std::vector<double>& Y) {
  Y.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) Y[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        double a = A[(size_t)i * m + j] * A[(size_t)i * m + j];
        tot += a;
        if (i != j) off += a;
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        double apq = A[(size_t)p * m + q];
        if (apq == 0.0) continue;
        double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
        double tau = (aqq - app) / (2.0 * apq);
        double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < m; ++k) {
          double akp = A[(size_t)k * m + p], akq = A[(size_t)k * m + q];
          A[(size_t)k * m + p] = c * akp - s * akq;
          A[(size_t)k * m + q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          double apk = A[(size_t)p * m + k], aqk = A[(size_t)q * m + k];
          A[(size_t)p * m + k] = c * apk - s * aqk;
          A[(size_t)q * m + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          double ykp = Y[(size_t)k * m + p], ykq = Y[(size_t)k * m + q];
          Y[(size_t)k * m + p] = c * ykp - s * ykq;
          Y[(size_t)k * m + q] = s * ykp + c * ykq;
        }
      }
  }
  std::vector<int> idx(m);
  for (int i = 0; i < m; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(),
                   [&](int a, int b) { return A[(size_t)a * m + a] < A[(size_t)b * m + b]; });
  theta.resize(m);
  std::vector<double> Ys((size_t)m * m);
  for (int c = 0; c < m; ++c) {
    theta[c] = A[(size_t)idx[c] * m + idx[c]];
    for (int r = 0; r < m; ++r) Ys[(size_t)r * m + c] = Y[(size_t)r * m + idx[c]];
  }
  Y.swap(Ys);
}

static void eps_free(ed_eps* e) {
  // a fixed-point copy made with one of these columns must not outlive them
  if (e->h && e->pool_r && e->h->xq_src) e->h->xq_src = nullptr;
  if (e->pool) cudaFree(e->pool);
  if (e->w) cudaFree(e->w);
  if (e->pool_r) cudaFree(e->pool_r);
  if (e->w_r) cudaFree(e->w_r);
  e->pool = nullptr;
  e->w = nullptr;
  e->pool_r = nullptr;
  e->w_r = nullptr;
  e->col.clear();
  e->col_r.clear();
  e->real_storage = false;
  e->pool_cols = 0;
}

// Orthogonalise w = H v_j against V[0..j].  First the local Lanczos
// projection (alpha = v_j^H w, and beta_{j-1} v_{j-1} when v_{j-1} is the
// previous Lanczos vector, i.e. j > k), fused with the dot products of one
// classical Gram-Schmidt pass against all of V[0..j]; then the CGS update,
// and a second CGS pass only if the norm fell below eta = 1/sqrt(2) of its
// value after the local projection (the DGKS criterion SLEPc applies by
// default).  In exact arithmetic this is the same projection as plain CGS;
// the local step removes the two large Lanczos components before the
// refinement test, so the second pass is needed only when real cancellation
// occurs.  h receives the total j+1 coefficients; norig = ||H v_j||.
//
// Real mode: H is real symmetric, so when the start vector is real (all
// imaginary parts exactly zero) every H.v, projection, normalisation and
// restart keeps the basis exactly real in complex128 arithmetic, and every
// coefficient v_i^H w has an exactly zero imaginary part.  The kernels then
// skip the products whose factors are those zeros (half the FP64 work) and
// give the same values as the full complex form.  A complex start vector
// (EPSSetInitialSpace) runs the full complex form.  (Keeping only Re(v_i^H w)
// for a complex start vector would be wrong in floating point: rounding
// seeds components along i*y for converged Ritz vectors y, which real
// coefficients never remove, and Lanczos then grows them into ghost copies.)
static int orthogonalize_lanczos(ed_eps* e, int j, int k, double beta_prev, std::vector<double2>& h, double* nw,
                                 double* norig, const double2* pre_a, double pre_y2) {
  ed_ctx* ctx = e->h->ctx;
  const int64_t n = e->h->basis->dim;
  std::vector<const double2*> cols(e->col.begin(), e->col.begin() + j + 1);
  h.assign(j + 1, make_double2(0.0, 0.0));
  double2 a;
  double y2 = 0.0, w2 = 0.0, n2 = 0.0;
  if (pre_a) {  // alpha = v_j^H w and ||w||^2 came with the H.v
    a = *pre_a;
    y2 = pre_y2;
  } else {
    ED_TRY(ed_multidot(ctx, &cols[j], 1, e->w, n, &a, &y2, e->real_coeffs));
  }
  *norig = std::sqrt(y2);
  const bool real = e->real_coeffs;
  if (real) a.y = 0.0;
  const bool three_term = j > k && j > 0;
  std::vector<double2> c(j + 1);
  ED_TRY(ed_local_multidot(ctx, cols.data(), j + 1, e->w, n, e->col[j], a, three_term ? e->col[j - 1] : nullptr,
                           beta_prev, c.data(), &w2, real));
  double n0 = std::sqrt(w2);
  h[j].x += a.x;
  h[j].y += a.y;
  if (three_term) h[j - 1].x += beta_prev;
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      ED_TRY(ed_multidot(ctx, cols.data(), j + 1, e->w, n, c.data(), nullptr, real));
    }
    ED_TRY(ed_update(ctx, cols.data(), j + 1, c.data(), e->w, n, &n2, real));
    for (int i = 0; i <= j; ++i) { h[i].x += c[i].x; h[i].y += c[i].y; }
    *nw = std::sqrt(n2);
    e->ortho_passes++;
    if (*nw >= 0.7071067811865476 * n0) break;
    n0 = *nw;
  }
  return ED_OK;
}

// Plain CGS with one conditional refinement (used for the random vector
// after an invariant subspace is found).
static int orthogonalize(ed_eps* e, int j, std::vector<double2>& h, double* nw, double* norig) {
  ed_ctx* ctx = e->h->ctx;
  const int64_t n = e->h->basis->dim;
  std::vector<const double2*> cols(e->col.begin(), e->col.begin() + j + 1);
  h.assign(j + 1, make_double2(0.0, 0.0));
  std::vector<double2> c(j + 1);
  double w2 = 0.0, n2 = 0.0;
  ED_TRY(ed_multidot(ctx, cols.data(), j + 1, e->w, n, c.data(), &w2));
  double n0 = std::sqrt(w2);
  *norig = n0;
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) ED_TRY(ed_multidot(ctx, cols.data(), j + 1, e->w, n, c.data(), nullptr));
    ED_TRY(ed_update(ctx, cols.data(), j + 1, c.data(), e->w, n, &n2));
    for (int i = 0; i <= j; ++i) { h[i].x += c[i].x; h[i].y += c[i].y; }
    *nw = std::sqrt(n2);
    if (*nw >= 0.7071067811865476 * n0) break;
    n0 = *nw;
  }
  return ED_OK;
}

// ---------------------------------------------------------------------------
// Real storage.  With a real start vector and H real symmetric the whole
// Krylov-Schur run has exactly zero imaginary parts (real mode, above); the
// basis then keeps only its real parts, which halves its memory and the
// traffic of every projection, update and restart.  The steps are those of
// orthogonalize_lanczos / eps_solve_impl; only the storage differs.
// ---------------------------------------------------------------------------
// *wmax: max_r |w_r| after the last pass, low 32 bits cleared.
static int orthogonalize_lanczos_r(ed_eps* e, int j, int k, double beta_prev, double a, double y2,
                                   std::vector<double>& h, double* nw, double* norig, double* wmax) {
  ed_ctx* ctx = e->h->ctx;
  const int64_t n = e->h->basis->dim;
  std::vector<const double*> cols(e->col_r.begin(), e->col_r.begin() + j + 1);
  h.assign(j + 1, 0.0);
  *norig = std::sqrt(y2);
  const bool three_term = j > k && j > 0;
  std::vector<double> c(j + 1);
  double n2 = 0.0;
  // no norm in the projection pass (one FP64 FMA per row less on the FP64
  // bound kernel): the norm before the update is sqrt(||w_after||^2 + sum c_i^2)
  // (Pythagoras against the orthonormal basis), formed after the update
  const bool exact = e->restart_mode == ED_RESTART_EXACT;
  const double margin = 1.0 + 0x1p-40;  // rounding of the bounds themselves
  int rc = ED_ENOTSUP;
  if (exact) {
    // max |w - a v_j - b v_j-1| <= ||w|| + |a| + |b| (unit columns)
    const double bound = (std::sqrt(y2) + std::fabs(a) + (three_term ? std::fabs(beta_prev) : 0.0)) * margin;
    rc = ed_multidot_tc(ctx, cols.data(), j + 1, e->w_r, n, e->col_r[j], a, three_term ? e->col_r[j - 1] : nullptr,
                        beta_prev, bound, c.data());
    if (rc == ED_ENOTSUP)  // the local step is done; the dots again in FP64
      rc = ed_multidot_r(ctx, cols.data(), j + 1, e->w_r, n, nullptr, 0.0, nullptr, 0.0, c.data(), nullptr);
  } else {
    rc = ed_multidot_r(ctx, cols.data(), j + 1, e->w_r, n, e->col_r[j], a, three_term ? e->col_r[j - 1] : nullptr,
                       beta_prev, c.data(), nullptr);
  }
  ED_TRY(rc);
  double n0 = -1.0;
  h[j] += a;
  if (three_term) h[j - 1] += beta_prev;
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      int r2 = ED_ENOTSUP;
      if (exact)
        r2 = ed_multidot_tc(ctx, cols.data(), j + 1, e->w_r, n, nullptr, 0.0, nullptr, 0.0, std::sqrt(n2) * margin,
                            c.data());
      if (r2 == ED_ENOTSUP)
        r2 = ed_multidot_r(ctx, cols.data(), j + 1, e->w_r, n, nullptr, 0.0, nullptr, 0.0, c.data(), nullptr);
      ED_TRY(r2);
    }
    ED_TRY(ed_update_r(ctx, cols.data(), j + 1, c.data(), e->w_r, n, &n2, wmax, e->restart_mode));
    for (int i = 0; i <= j; ++i) h[i] += c[i];
    *nw = std::sqrt(n2);
    if (n0 < 0.0) {
      double s2 = n2;
      for (int i = 0; i <= j; ++i) s2 += c[i] * c[i];
      n0 = std::sqrt(s2);
    }
    e->ortho_passes++;
    if (*nw >= 0.7071067811865476 * n0) break;
    n0 = *nw;
  }
  return ED_OK;
}

static int orthogonalize_r(ed_eps* e, int j, double* nw) {
  ed_ctx* ctx = e->h->ctx;
  const int64_t n = e->h->basis->dim;
  std::vector<const double*> cols(e->col_r.begin(), e->col_r.begin() + j + 1);
  std::vector<double> c(j + 1);
  double w2 = 0.0, n2 = 0.0;
  ED_TRY(ed_multidot_r(ctx, cols.data(), j + 1, e->w_r, n, nullptr, 0.0, nullptr, 0.0, c.data(), &w2));
  double n0 = std::sqrt(w2);
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1)
      ED_TRY(ed_multidot_r(ctx, cols.data(), j + 1, e->w_r, n, nullptr, 0.0, nullptr, 0.0, c.data(), nullptr));
    ED_TRY(ed_update_r(ctx, cols.data(), j + 1, c.data(), e->w_r, n, &n2, nullptr, e->restart_mode));
    *nw = std::sqrt(n2);
    if (*nw >= 0.7071067811865476 * n0) break;
    n0 = *nw;
  }
  return ED_OK;
}

static int eps_solve_real(ed_eps* e, int* nconv_out, int m, int nev, double tol, int max_it) {
  ed_ham* H = e->h;
  ed_ctx* ctx = H->ctx;
  const int64_t n = H->basis->dim;
  // float pairs and exact slices only on request; the default keeps every
  // product at FP64 or better (FP64 FMA beside exact integers)
  e->restart_mode = e->restart_arith == ED_RESTART_AUTO ? ED_RESTART_FP64 : e->restart_arith;
  if (e->restart_mode == ED_RESTART_EXACT && m > 32)
    return ed_fail(ED_ENOTSUP, "the exact tensor-core restart takes at most 32 basis vectors (ncv <= 32)");
  e->pool_cols = 2 * m + 1;
  if (cudaMalloc(&e->pool_r, sizeof(double) * (size_t)n * e->pool_cols) != cudaSuccess ||
      cudaMalloc(&e->w_r, sizeof(double) * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    eps_free(e);
    return ed_fail(ED_ENOMEM, "Krylov basis does not fit in device memory");
  }
  e->real_storage = true;
  e->real_coeffs = true;
  std::vector<double*> freelist;
  e->col_r.assign(m + 1, nullptr);
  for (int i = 0; i < e->pool_cols; ++i) {
    double* p = e->pool_r + (size_t)i * n;
    if (i <= m) e->col_r[i] = p; else freelist.push_back(p);
  }
  std::vector<double> alpha(m + 1, 0.0), beta(m + 1, 0.0), arrow(m + 1, 0.0);
  if (e->v0) ED_TRY(ed_complex_to_real(ctx, e->v0, e->col_r[0], n));
  else ED_TRY(ed_start_vector_r(ctx, e->seed, n, e->col_r[0]));
  {
    double v2 = 0.0;
    ED_TRY(ed_multidot_r(ctx, nullptr, 0, e->col_r[0], n, nullptr, 0.0, nullptr, 0.0, nullptr, &v2));
    ED_TRY(ed_scale_copy_r(ctx, e->col_r[0], e->col_r[0], 1.0 / std::sqrt(v2), n));
  }
  uint64_t rseed = e->seed + 0x51ED2701ull;
  e->nhv = 0;
  e->ortho_passes = 0;
  int k = 0, nconv = 0, its = 0;
  std::vector<double> theta, Y, h;
  bool done = false;
  while (!done) {
    ++its;
    for (int j = k; j < m; ++j) {
      double2 pre_a;
      double pre_y2 = 0.0;
      ED_TRY(ed_launch_hv_dot_any(H, e->col_r[j], e->w_r, true, &pre_a, &pre_y2));
      e->nhv++;
      double nw = 0.0, norig = 0.0, wmax = 0.0;
      ED_TRY(orthogonalize_lanczos_r(e, j, k, j > 0 ? beta[j - 1] : 0.0, pre_a.x, pre_y2, h, &nw, &norig, &wmax));
      alpha[j] = h[j];
      if (nw <= 1e-13 * norig) {
        // invariant subspace: continue with a (real) random vector orthogonal to V
        beta[j] = 0.0;
        if (j + 1 < m) {
          ED_TRY(ed_start_vector_r(ctx, rseed++, n, e->w_r));
          double nw2 = 0.0;
          ED_TRY(orthogonalize_r(e, j, &nw2));
          ED_TRY(ed_scale_copy_r(ctx, e->w_r, e->col_r[j + 1], 1.0 / nw2, n));
        } else {
          ED_CUDA(cudaMemsetAsync(e->col_r[j + 1], 0, sizeof(double) * (size_t)n, ctx->stream));
        }
      } else {
        // the next H.v's input is this vector: its fixed-point copy is made in
        // the same pass (bit-identical to quantizing it afterwards)
        const int rq = ed_scale_quantize_r(H, e->w_r, e->col_r[j + 1], 1.0 / nw, wmax);
        if (rq == ED_ENOTSUP) ED_TRY(ed_scale_copy_r(ctx, e->w_r, e->col_r[j + 1], 1.0 / nw, n));
        else if (rq != ED_OK) return rq;
        beta[j] = nw;
      }
    }
    std::vector<double> T((size_t)m * m, 0.0);
    for (int i = 0; i < k; ++i) {
      T[(size_t)i * m + i] = alpha[i];
      T[(size_t)i * m + k] = T[(size_t)k * m + i] = arrow[i];
    }
    for (int j = k; j < m; ++j) {
      T[(size_t)j * m + j] = alpha[j];
      if (j + 1 < m) T[(size_t)j * m + j + 1] = T[(size_t)(j + 1) * m + j] = beta[j];
    }
    ed_jacobi_eig(m, T, theta, Y);
    const double bm = beta[m - 1];
    nconv = 0;
    for (int i = 0; i < m; ++i) {
      double res = std::fabs(bm * Y[(size_t)(m - 1) * m + i]);
      double rel = res / std::max(std::fabs(theta[i]), 1e-300);
      if (rel < tol) ++nconv; else break;
    }
    if (nconv >= nev || its >= max_it) done = true;
    int l;
    if (done) l = std::min(m, std::max(nconv, nev));
    else {
      l = nconv + std::max(1, (m - nconv) / 2);
      if (l > m - 1) l = m - 1;
    }
    std::vector<double*> outc(freelist.begin(), freelist.begin() + l);
    std::vector<const double*> inc(e->col_r.begin(), e->col_r.begin() + m);
    ED_TRY(ed_restart_combine_r(ctx, inc.data(), m, Y.data(), m, l, outc.data(), n, e->restart_mode));
    std::vector<double*> newcol(m + 1, nullptr);
    for (int c = 0; c < l; ++c) newcol[c] = outc[c];
    newcol[l] = e->col_r[m];
    std::vector<double*> newfree(freelist.begin() + l, freelist.end());
    for (int c = 0; c < m; ++c) newfree.push_back(e->col_r[c]);
    for (int c = l + 1; c <= m; ++c) { newcol[c] = newfree.back(); newfree.pop_back(); }
    e->col_r.swap(newcol);
    freelist.swap(newfree);
    if (done) {
      e->nrep = l;
      e->nconv = std::min(nconv, l);
      e->evals.assign(theta.begin(), theta.begin() + l);
      e->errs.assign(l, 0.0);
      for (int c = 0; c < l; ++c) {
        ED_TRY(ed_launch_hv_r(H, e->col_r[c], e->w_r));
        double r2, x2;
        ED_TRY(ed_residual_norm2_r(ctx, e->w_r, e->col_r[c], theta[c], n, &r2, &x2));
        e->errs[c] = std::sqrt(r2) / std::max(std::fabs(theta[c]) * std::sqrt(x2), 1e-300);
      }
      break;
    }
    for (int i = 0; i < l; ++i) { alpha[i] = theta[i]; arrow[i] = bm * Y[(size_t)(m - 1) * m + i]; }
    k = l;
  }
  e->its = its;
  e->solved = true;
  *nconv_out = e->nconv;
  return ED_OK;
}

static int eps_solve_impl(ed_eps* e, int* nconv_out) {
  ed_ham* H = e->h;
  ed_ctx* ctx = H->ctx;
  const int64_t n = H->basis->dim;
  int nev = e->nev;
  int ncv = e->ncv > 0 ? e->ncv : std::max(2 * nev, nev + 15);
  if (ncv > n) ncv = (int)n;
  if (nev > ncv) nev = ncv;
  if (ncv > 126) return ed_fail(ED_ENOTSUP, "ncv above 126 is not supported");
  const double tol = e->tol > 0 ? e->tol : 1e-8;
  const int max_it = e->max_it > 0 ? e->max_it : (int)std::max<int64_t>(100, 2 * n / std::max(ncv, 1));
  const int m = ncv;
  eps_free(e);
  {
    bool real_start = true;
    if (e->v0) ED_TRY(ed_is_real(ctx, e->v0, n, &real_start));
    if (real_start && ed_lin_supported(H)) return eps_solve_real(e, nconv_out, m, nev, tol, max_it);
  }
  e->pool_cols = 2 * m + 1;
  if (cudaMalloc(&e->pool, sizeof(double2) * (size_t)n * e->pool_cols) != cudaSuccess ||
      cudaMalloc(&e->w, sizeof(double2) * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    eps_free(e);
    return ed_fail(ED_ENOMEM, "Krylov basis does not fit in device memory");
  }
  std::vector<double2*> freelist;
  e->col.assign(m + 1, nullptr);
  for (int i = 0; i < e->pool_cols; ++i) {
    double2* p = e->pool + (size_t)i * n;
    if (i <= m) e->col[i] = p; else freelist.push_back(p);
  }
  std::vector<double> alpha(m + 1, 0.0), beta(m + 1, 0.0), arrow(m + 1, 0.0);
  // start vector: the user's (EPSSetInitialSpace) or the seeded one
  bool real_start = true;
  if (e->v0) {
    ED_TRY(ed_copy(ctx, e->v0, e->col[0], n));
    ED_TRY(ed_is_real(ctx, e->v0, n, &real_start));
  } else {
    ED_TRY(ed_start_vector(ctx, e->seed, n, e->col[0], true));
  }
  {
    std::vector<double2> none;
    double v2 = 0.0;
    ED_TRY(ed_multidot(ctx, nullptr, 0, e->col[0], n, none.data(), &v2));
    ED_TRY(ed_scale_copy(ctx, e->col[0], e->col[0], 1.0 / std::sqrt(v2), n));
  }
  uint64_t rseed = e->seed + 0x51ED2701ull;
  e->nhv = 0;
  e->ortho_passes = 0;
  e->real_coeffs = real_start;
  int k = 0, nconv = 0, its = 0;
  std::vector<double> theta, Y;
  std::vector<double2> h;
  bool done = false;
  while (!done) {
    ++its;
    for (int j = k; j < m; ++j) {
      double2 pre_a = make_double2(0.0, 0.0);
      double pre_y2 = 0.0;
      bool fused = false;
      if (ed_lin_supported(H)) {
        ED_TRY(ed_launch_hv_dot(H, e->col[j], e->w, &pre_a, &pre_y2));
        fused = true;
      } else {
        ED_TRY(ed_launch_hv(H, e->col[j], e->w));
      }
      e->nhv++;
      double nw = 0.0, norig = 0.0;
      ED_TRY(orthogonalize_lanczos(e, j, k, j > 0 ? beta[j - 1] : 0.0, h, &nw, &norig, fused ? &pre_a : nullptr,
                                   pre_y2));
      alpha[j] = h[j].x;
      if (nw <= 1e-13 * norig) {
        // invariant subspace: continue with a random vector orthogonal to V
        beta[j] = 0.0;
        if (j + 1 < m) {
          ED_TRY(ed_start_vector(ctx, rseed++, n, e->w, e->real_coeffs));
          std::vector<double2> h2;
          double nw2 = 0.0, no2 = 0.0;
          ED_TRY(orthogonalize(e, j, h2, &nw2, &no2));
          ED_TRY(ed_scale_copy(ctx, e->w, e->col[j + 1], 1.0 / nw2, n));
        } else {
          ED_CUDA(cudaMemsetAsync(e->col[j + 1], 0, sizeof(double2) * (size_t)n, ctx->stream));
        }
      } else {
        ED_TRY(ed_scale_copy(ctx, e->w, e->col[j + 1], 1.0 / nw, n));
        beta[j] = nw;
      }
    }
    std::vector<double> T((size_t)m * m, 0.0);
    for (int i = 0; i < k; ++i) {
      T[(size_t)i * m + i] = alpha[i];
      T[(size_t)i * m + k] = T[(size_t)k * m + i] = arrow[i];
    }
    for (int j = k; j < m; ++j) {
      T[(size_t)j * m + j] = alpha[j];
      if (j + 1 < m) T[(size_t)j * m + j + 1] = T[(size_t)(j + 1) * m + j] = beta[j];
    }
    ed_jacobi_eig(m, T, theta, Y);
    const double bm = beta[m - 1];
    nconv = 0;
    for (int i = 0; i < m; ++i) {
      double res = std::fabs(bm * Y[(size_t)(m - 1) * m + i]);
      double rel = res / std::max(std::fabs(theta[i]), 1e-300);
      if (rel < tol) ++nconv; else break;
    }
    if (nconv >= nev || its >= max_it) done = true;
    int l;
    if (done) l = std::min(m, std::max(nconv, nev));
    else {
      l = nconv + std::max(1, (m - nconv) / 2);
      if (l > m - 1) l = m - 1;
    }
    // new columns 0..l-1 = V Y[:, 0..l-1] into free columns
    std::vector<double2*> outc(freelist.begin(), freelist.begin() + l);
    std::vector<const double2*> inc(e->col.begin(), e->col.begin() + m);
    ED_TRY(ed_restart_combine(ctx, inc.data(), m, Y.data(), m, l, outc.data(), n, e->real_coeffs));
    std::vector<double2*> newcol(m + 1, nullptr);
    for (int c = 0; c < l; ++c) newcol[c] = outc[c];
    newcol[l] = e->col[m];
    std::vector<double2*> newfree(freelist.begin() + l, freelist.end());
    for (int c = 0; c < m; ++c) newfree.push_back(e->col[c]);
    for (int c = l + 1; c <= m; ++c) { newcol[c] = newfree.back(); newfree.pop_back(); }
    e->col.swap(newcol);
    freelist.swap(newfree);
    if (done) {
      e->nrep = l;
      e->nconv = std::min(nconv, l);
      e->evals.assign(theta.begin(), theta.begin() + l);
      e->errs.assign(l, 0.0);
      for (int c = 0; c < l; ++c) {
        ED_TRY(ed_launch_hv(H, e->col[c], e->w));
        double r2, x2;
        ED_TRY(ed_residual_norm2(ctx, e->w, e->col[c], theta[c], n, &r2, &x2));
        e->errs[c] = std::sqrt(r2) / std::max(std::fabs(theta[c]) * std::sqrt(x2), 1e-300);
      }
      break;
    }
    for (int i = 0; i < l; ++i) { alpha[i] = theta[i]; arrow[i] = bm * Y[(size_t)(m - 1) * m + i]; }
    k = l;
  }
  e->its = its;
  e->solved = true;
  *nconv_out = e->nconv;
  return ED_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int ed_eps_create(ed_ham* h, int nev, int ncv, int mpd, ed_eps** out) {
  if (!h || !out) return ed_fail(ED_EINVAL, "null argument");
  if (nev < 1) return ed_fail(ED_EINVAL, "nev must be >= 1");
  ed_eps* e = new ed_eps();
  e->h = h;
  e->nev = nev;
  e->ncv = ncv;
  e->mpd = mpd;
  *out = e;
  return ED_OK;
}

int ed_eps_set_dimensions(ed_eps* e, int nev, int ncv, int mpd) {
  if (!e) return ed_fail(ED_EINVAL, "null solver");
  if (nev < 1) return ed_fail(ED_EINVAL, "nev must be >= 1");
  e->nev = nev;
  e->ncv = ncv;
  e->mpd = mpd;
  return ED_OK;
}

int ed_eps_set_tolerances(ed_eps* e, double tol, int max_it) {
  if (!e) return ed_fail(ED_EINVAL, "null solver");
  e->tol = tol;
  e->max_it = max_it;
  return ED_OK;
}

int ed_eps_set_seed(ed_eps* e, uint64_t seed) {
  if (!e) return ed_fail(ED_EINVAL, "null solver");
  e->seed = seed;
  return ED_OK;
}

int ed_eps_set_restart_arithmetic(ed_eps* e, int mode) {
  if (!e) return ed_fail(ED_EINVAL, "null solver");
  if (mode != ED_RESTART_AUTO && mode != ED_RESTART_FP64 && mode != ED_RESTART_PAIR && mode != ED_RESTART_EXACT &&
      mode != ED_RESTART_FIXED)
    return ed_fail(ED_EINVAL, "unknown restart arithmetic");
  e->restart_arith = mode;
  return ED_OK;
}

int ed_eps_set_initial_vector(ed_eps* e, const ed_cplx* v, int on_device) {
  if (!e) return ed_fail(ED_EINVAL, "null solver");
  ed_ctx* ctx = e->h->ctx;
  if (!v) {
    if (e->v0) cudaFree(e->v0);
    e->v0 = nullptr;
    return ED_OK;
  }
  const size_t bytes = sizeof(double2) * (size_t)e->h->basis->dim;
  if (!e->v0) ED_CUDA(cudaMalloc(&e->v0, bytes));
  ED_CUDA(cudaMemcpyAsync(e->v0, v, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  return ED_OK;
}

int ed_eps_solve(ed_eps* e, int* nconv) {
  if (!e || !nconv) return ed_fail(ED_EINVAL, "null argument");
  if (!e->h->d_diag) return ed_fail(ED_ESTATE, "Hamiltonian has no assembled diagonal");
  int rc = eps_solve_impl(e, nconv);
  if (rc == ED_OK && e->nconv < std::min(e->nev, (int)e->h->basis->dim)) {
    // like EPSSolve: not an error, nconv reports what converged
  }
  return rc;
}

int ed_eps_get_eigenpair(ed_eps* e, int i, double* eig, double* rel_err, ed_cplx* vec_dev) {
  if (!e) return ed_fail(ED_EINVAL, "null solver");
  if (!e->solved) return ed_fail(ED_ESTATE, "eigenpair requested before solve");
  if (i < 0 || i >= e->nrep) return ed_fail(ED_EINVAL, "eigenpair index out of range");
  if (eig) *eig = e->evals[i];
  if (rel_err) *rel_err = e->errs[i];
  if (vec_dev) {
    if (e->real_storage) ED_TRY(ed_real_to_complex(e->h->ctx, e->col_r[i], (double2*)vec_dev, e->h->basis->dim));
    else ED_TRY(ed_copy(e->h->ctx, e->col[i], (double2*)vec_dev, e->h->basis->dim));
  }
  return ED_OK;
}

int ed_eps_get_eigenvector_host(ed_eps* e, int i, ed_cplx* vec_host) {
  if (!e || !vec_host) return ed_fail(ED_EINVAL, "null argument");
  if (!e->solved) return ed_fail(ED_ESTATE, "eigenvector requested before solve");
  if (i < 0 || i >= e->nrep) return ed_fail(ED_EINVAL, "eigenpair index out of range");
  ed_ctx* ctx = e->h->ctx;
  const int64_t n = e->h->basis->dim;
  if (e->real_storage) {
    // expand to complex128 in halves through a basis column that holds no
    // Ritz vector (col_r[m], n doubles = n/2 complex entries) and the work
    // vector: no allocation
    const int m = (int)e->col_r.size() - 1;
    if (n < 2) {  // one state: a column cannot hold one complex entry
      double v = 0.0;
      ED_CUDA(cudaMemcpyAsync(&v, e->col_r[i], sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      ED_CUDA(cudaStreamSynchronize(ctx->stream));
      std::memcpy(vec_host, &v, sizeof(double));
      std::memset((char*)vec_host + sizeof(double), 0, sizeof(double));
      return ED_OK;
    }
    // two stages (that column and the work vector, both free after the
    // solve): both halves are expanded and copied back with one wait
    double2* stage[2] = {(double2*)e->col_r[m], (double2*)e->w_r};
    const int64_t half = n / 2;  // complex entries a stage holds
    int q = 0;
    for (int64_t r0 = 0; r0 < n; r0 += half, ++q) {
      if (q >= 2) ED_CUDA(cudaStreamSynchronize(ctx->stream));  // odd n: a third chunk reuses a stage
      const int64_t c = std::min(half, n - r0);
      ED_TRY(ed_real_to_complex(ctx, e->col_r[i] + r0, stage[q & 1], c));
      ED_CUDA(cudaMemcpyAsync(vec_host + r0, stage[q & 1], sizeof(double2) * (size_t)c, cudaMemcpyDeviceToHost,
                              ctx->stream));
    }
    ED_CUDA(cudaStreamSynchronize(ctx->stream));
    return ED_OK;
  }
  ED_CUDA(cudaMemcpyAsync(vec_host, e->col[i], sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
  ED_CUDA(cudaStreamSynchronize(ctx->stream));
  return ED_OK;
}

int ed_eps_get_stats(ed_eps* e, int* its, int64_t* n_hv, int* n_reported, int64_t* ortho_passes) {
  if (!e) return ed_fail(ED_EINVAL, "null solver");
  if (ortho_passes) *ortho_passes = e->ortho_passes;
  if (its) *its = e->its;
  if (n_hv) *n_hv = e->nhv;
  if (n_reported) *n_reported = e->nrep;
  return ED_OK;
}

int ed_eps_destroy(ed_eps* e) {
  if (!e) return ED_OK;
  eps_free(e);
  if (e->v0) cudaFree(e->v0);
  delete e;
  return ED_OK;
}

}  // extern "C"
