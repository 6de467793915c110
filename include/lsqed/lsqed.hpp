// lsqed.hpp — header-only C++ shim that re-creates LSQuantumED's hot-path
// class interfaces on top of the C ABI in ed_capi.h, with the PETSc handle
// types the reference's drivers use: Mat (Hamiltonian<L>::hamilt), Vec
// (device vectors from MatCreateVecs, freed by VecDestroy) and EPS.  PETSc
// types map as: PetscInt -> int64_t, PetscReal -> double, PetscScalar ->
// lsqed::Scalar (complex, converting to its real part where a double is
// expected, as PETSc's C complex scalars do in C++), PetscErrorCode -> int.
// lsqed_dropin.hpp adds the global names, option parsing and logging calls
// so that the reference's drivers (examples/main.cpp, main_disorder.cpp,
// ex1-4.cpp) compile with only their #include lines replaced.
//
// Link with -ledgb300 (lsquantumed_gb300/_lib/libedgb300.so).
#pragma once
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "../ed_capi.h"

namespace lsqed {

typedef int64_t PetscInt;
typedef double PetscReal;
typedef int PetscErrorCode;
enum PetscBool { PETSC_FALSE = 0, PETSC_TRUE = 1 };
static const PetscInt PETSC_DECIDE = -1;
static const PetscInt PETSC_DEFAULT = -2;

// Complex scalar (complex128).  It converts implicitly to double (its real
// part) and from double, and mixes with double in arithmetic, like PETSc's
// C complex scalars in C++ code: drivers written for real and for complex
// PETSc builds compile against it unchanged.
struct Scalar {
  double re = 0.0, im = 0.0;
  Scalar() {}
  Scalar(double r) : re(r) {}
  Scalar(double r, double i) : re(r), im(i) {}
  Scalar(const std::complex<double>& z) : re(z.real()), im(z.imag()) {}
  operator double() const { return re; }
  std::complex<double> c() const { return std::complex<double>(re, im); }
  double real() const { return re; }
  double imag() const { return im; }
  Scalar& operator+=(const Scalar& o) { re += o.re; im += o.im; return *this; }
  Scalar& operator-=(const Scalar& o) { re -= o.re; im -= o.im; return *this; }
  Scalar& operator*=(const Scalar& o) { *this = Scalar(c() * o.c()); return *this; }
  Scalar& operator/=(const Scalar& o) { *this = Scalar(c() / o.c()); return *this; }
  Scalar& operator+=(double o) { re += o; return *this; }
  Scalar& operator-=(double o) { re -= o; return *this; }
  Scalar& operator*=(double o) { re *= o; im *= o; return *this; }
  Scalar& operator/=(double o) { re /= o; im /= o; return *this; }
};
inline Scalar operator+(Scalar a, const Scalar& b) { return a += b; }
inline Scalar operator-(Scalar a, const Scalar& b) { return a -= b; }
inline Scalar operator*(Scalar a, const Scalar& b) { return a *= b; }
inline Scalar operator/(Scalar a, const Scalar& b) { return a /= b; }
inline Scalar operator+(Scalar a, double b) { return a += b; }
inline Scalar operator-(Scalar a, double b) { return a -= b; }
inline Scalar operator*(Scalar a, double b) { return a *= b; }
inline Scalar operator/(Scalar a, double b) { return a /= b; }
inline Scalar operator+(double a, const Scalar& b) { return Scalar(a) += b; }
inline Scalar operator-(double a, const Scalar& b) { return Scalar(a) -= b; }
inline Scalar operator*(double a, const Scalar& b) { return Scalar(a) *= b; }
inline Scalar operator/(double a, const Scalar& b) { return Scalar(a) /= b; }
inline Scalar operator+(Scalar a, int b) { return a += (double)b; }
inline Scalar operator*(Scalar a, int b) { return a *= (double)b; }
inline Scalar operator/(Scalar a, int b) { return a /= (double)b; }
inline Scalar operator/(Scalar a, PetscInt b) { return a /= (double)b; }
inline Scalar operator-(const Scalar& a) { return Scalar(-a.re, -a.im); }
typedef Scalar PetscScalar;
inline double PetscRealPart(const Scalar& z) { return z.re; }
inline double PetscRealPart(double x) { return x; }
inline double PetscImaginaryPart(const Scalar& z) { return z.im; }
inline double PetscImaginaryPart(double) { return 0.0; }

inline std::string last_error() {
  char buf[1024];
  ed_last_error(buf, sizeof(buf));
  return buf;
}

// Map C ABI status to the reference's behaviour: constructors throw
// std::invalid_argument / std::runtime_error, other calls return codes.
inline void throw_on(int rc) {
  if (rc == ED_OK) return;
  if (rc == ED_EINVAL) throw std::invalid_argument(last_error());
  throw std::runtime_error(last_error());
}
#define ED_TRY_SHIM(expr)           \
  do {                              \
    int _rc = (expr);               \
    if (_rc != ED_OK) return _rc;   \
  } while (0)

// ---------------------------------------------------------------------------
// Environment (include/environment.hpp:20-53)
// ---------------------------------------------------------------------------
// The solver options of the command line, as PETSc's options database holds
// them for EPSSetFromOptions (src/solver.cpp:21): -eps_tol and -eps_max_it
// apply to every solver SolverInit creates, the DSF one included.
struct SolverOptions {
  double eps_tol = 0.0;  // 0: the library default (1e-8)
  int eps_max_it = 0;    // 0: the library default
};
inline SolverOptions& solver_options() {
  static SolverOptions o;
  return o;
}
inline void parse_solver_options(int argc, char** argv) {
  if (!argv) return;
  for (int i = 1; i + 1 < argc; ++i) {
    std::string k = argv[i];
    for (auto& ch : k) ch = (char)((ch >= 'A' && ch <= 'Z') ? ch - 'A' + 'a' : ch);
    if (k == "-eps_tol") solver_options().eps_tol = std::atof(argv[i + 1]);
    else if (k == "-eps_max_it") solver_options().eps_max_it = std::atoi(argv[i + 1]);
  }
}

// The command line, kept for the option queries of the drivers (the
// reference's PETSc options database, filled by SlepcInitialize).
struct CommandLine {
  std::vector<std::string> args;
};
inline CommandLine& command_line() {
  static CommandLine c;
  return c;
}

class Environment {
 public:
  PetscInt nspins = 0;
  int mpi_rank = 0, mpi_size = 1;
  bool disorder_flg = false;
  ed_ctx* ctx = nullptr;

  Environment(int argc, char** argv, const char* /*help*/ = nullptr) { init(argc, argv); }
  Environment(int argc, char** argv, PetscInt m_nspins, const char* /*help*/ = nullptr) {
    if (m_nspins % 2 != 0) throw std::invalid_argument("The total number of spins has to be EVEN.");
    if (m_nspins <= 0) throw std::invalid_argument("The total number of spins has to be POSITIVE.");
    nspins = m_nspins;
    init(argc, argv);
  }
  ~Environment() { ed_ctx_destroy(ctx); }
  Environment(const Environment&) = delete;
  Environment& operator=(const Environment&) = delete;

 private:
  void init(int argc, char** argv) {
    command_line().args.assign(argv, argv + (argv ? argc : 0));
    parse_solver_options(argc, argv);
    if (ed_ctx_create(0, nullptr, &ctx) != ED_OK)
      throw std::runtime_error("Slepc was not correctly initialized\n" + last_error());
  }
};

// ---------------------------------------------------------------------------
// Basis (include/basis.hpp:67-93)
// ---------------------------------------------------------------------------
class Basis {
 public:
  PetscInt nspins, total_mag, nspins_up, max_mag, size, local_size, global_start_index;
  int mpi_size = 1, mpi_rank = 0;
  ed_basis* h = nullptr;

  Basis(Environment& env, PetscInt m_total_mag) {
    throw_on(ed_basis_create(env.ctx, (int)env.nspins, (int)m_total_mag, &h));
    int ns, nup, tm;
    int64_t sz;
    throw_on(ed_basis_info(h, &sz, &ns, &nup, &tm));
    nspins = ns; nspins_up = nup; total_mag = tm; max_mag = ns / 2;
    size = sz; local_size = sz; global_start_index = 0;
  }
  ~Basis() { ed_basis_destroy(h); }
  Basis(const Basis&) = delete;
  Basis& operator=(const Basis&) = delete;
  // int_basis (basis.cpp:192-215), fetched on demand
  std::vector<PetscInt> int_basis() const {
    std::vector<uint64_t> s((size_t)size);
    throw_on(ed_basis_states_host(h, 0, size, s.data()));
    return std::vector<PetscInt>(s.begin(), s.end());
  }
};

// ---------------------------------------------------------------------------
// Lattices (include/lattice.hpp:166-329)
// ---------------------------------------------------------------------------
class Lattice {
 public:
  PetscInt nspins, nspins_x, nspins_y;
  std::vector<int32_t> nn, nnn;  // flattened (i, j) pairs in visiting order
 protected:
  Lattice(Environment& env, int ltype, PetscInt lx, PetscInt ly) : nspins(env.nspins), nspins_x(lx), nspins_y(ly) {
    int64_t na = 0, nb = 0;
    throw_on(ed_lattice_bonds(ltype, (int)nspins, (int)lx, (int)ly, nullptr, 0, &na, nullptr, 0, &nb));
    nn.resize(2 * na);
    nnn.resize(2 * nb);
    throw_on(ed_lattice_bonds(ltype, (int)nspins, (int)lx, (int)ly, nn.data(), na, &na, nnn.data(), nb, &nb));
  }
 public:
  PetscInt num_spins() const { return nspins; }
};
class chain1D : public Lattice {
 public:
  explicit chain1D(Environment& env) : Lattice(env, ED_CHAIN1D, 1, env.nspins) {}
};
class square2D : public Lattice {
 public:
  square2D(Environment& env, PetscInt lx, PetscInt ly) : Lattice(env, ED_SQUARE2D, lx, ly) {}
};
class honeycomb2D : public Lattice {
 public:
  honeycomb2D(Environment& env, PetscInt lx, PetscInt ly) : Lattice(env, ED_HONEYCOMB2D, lx, ly) {}
};

// ---------------------------------------------------------------------------
// PETSc handles: Vec (a device vector of complex128 entries) and Mat (the
// Hamiltonian's matrix-free operator).  MatCreateVecs / VecDestroy follow
// PETSc's calling convention (src/solver.cpp, examples/*.cpp).
// ---------------------------------------------------------------------------
struct _p_Vec {
  ed_ctx* ctx = nullptr;
  ed_cplx* d = nullptr;
  PetscInt n = 0;
};
typedef _p_Vec* Vec;
struct _p_Mat {
  ed_ctx* ctx = nullptr;
  ed_ham* h = nullptr;
  PetscInt n = 0;
};
typedef _p_Mat* Mat;

inline PetscErrorCode VecCreateOnDevice(ed_ctx* ctx, PetscInt n, Vec* v) {
  Vec x = new _p_Vec();
  x->ctx = ctx;
  x->n = n;
  int rc = ed_vec_create(ctx, n, &x->d);
  if (rc != ED_OK) {
    delete x;
    return rc;
  }
  *v = x;
  return ED_OK;
}
// MatCreateVecs(mat, &right, &left): vectors the operator can act on / fill.
inline PetscErrorCode MatCreateVecs(Mat A, Vec* right, Vec* left) {
  if (!A) return ED_EINVAL;
  if (right) ED_TRY_SHIM(VecCreateOnDevice(A->ctx, A->n, right));
  if (left) ED_TRY_SHIM(VecCreateOnDevice(A->ctx, A->n, left));
  return ED_OK;
}
inline PetscErrorCode VecDestroy(Vec* v) {
  if (!v || !*v) return ED_OK;
  ed_vec_destroy((*v)->d);
  delete *v;
  *v = nullptr;
  return ED_OK;
}
inline PetscErrorCode VecGetSize(Vec v, PetscInt* n) {
  *n = v ? v->n : 0;
  return ED_OK;
}
// Host copies (VecGetArray with a copy back), for drivers that post-process.
inline std::vector<PetscScalar> VecToHost(Vec v) {
  std::vector<ed_cplx> tmp((size_t)v->n);
  throw_on(ed_vec_to_host(v->ctx, v->d, tmp.data(), v->n));
  std::vector<PetscScalar> out((size_t)v->n);
  for (size_t k = 0; k < tmp.size(); ++k) out[k] = PetscScalar(tmp[k].re, tmp[k].im);
  return out;
}

// ---------------------------------------------------------------------------
// Hamiltonian<L> (include/hamiltonian.hpp:187-299)
// ---------------------------------------------------------------------------
template <typename L>
class Hamiltonian {
 public:
  Mat hamilt = nullptr;  // the reference's `Mat hamilt` (hamiltonian.hpp:187)
  Basis& basis;
  L& lattice;
  PetscReal J1, Delta1, J2, Delta2;

  Hamiltonian(Environment& env, Basis& b, L& lat, PetscReal m_J1, PetscReal m_D1, PetscReal m_J2, PetscReal m_D2)
      : basis(b), lattice(lat), J1(m_J1), Delta1(m_D1), J2(m_J2), Delta2(m_D2) {
    hamilt = new _p_Mat();
    hamilt->ctx = env.ctx;
    hamilt->n = b.size;
    int rc = ed_ham_create(env.ctx, b.h, lat.nn.data(), (int64_t)lat.nn.size() / 2, lat.nnn.data(),
                           (int64_t)lat.nnn.size() / 2, J1, Delta1, J2, Delta2, &hamilt->h);
    if (rc != ED_OK) {
      delete hamilt;
      throw std::runtime_error("The matrix has not been properly initialized.\n" + last_error());
    }
  }
  ~Hamiltonian() {
    ed_ham_destroy(hamilt->h);
    delete hamilt;
  }
  Hamiltonian(const Hamiltonian&) = delete;
  Hamiltonian& operator=(const Hamiltonian&) = delete;

  PetscErrorCode build_diag(Environment&) { return ed_ham_build_diag(hamilt->h); }
  PetscErrorCode build_off_diag(Environment&) { return ed_ham_build_off_diag(hamilt->h); }
  PetscErrorCode build_disorder(Environment& env, PetscReal* hi) {
    env.disorder_flg = true;
    return ed_ham_build_disorder(hamilt->h, hi);
  }
  PetscInt hamilt_size() const { return basis.size; }
  PetscReal hamilt_J1() const { return J1; }
  PetscReal hamilt_J2() const { return J2; }
  PetscReal hamilt_D1() const { return Delta1; }
  PetscReal hamilt_D2() const { return Delta2; }
};

// ---------------------------------------------------------------------------
// Solver:: (include/solver.hpp:27-66)
// ---------------------------------------------------------------------------
struct EPS {
  ed_eps* e = nullptr;
};

namespace Solver {
// SolverInit(EPS&, Mat, nev, ncv, mpd) (include/solver.hpp:27-31):
// Hermitian, Krylov-Schur, smallest real; -eps_tol / -eps_max_it of the
// command line applied as EPSSetFromOptions would.
inline PetscErrorCode SolverInit(EPS& solver, Mat matrix, PetscInt nev, PetscInt ncv = PETSC_DEFAULT,
                                 PetscInt mpd = PETSC_DEFAULT) {
  if (!matrix) return ED_EINVAL;
  PetscErrorCode rc = ed_eps_create(matrix->h, (int)nev, (int)ncv, (int)mpd, &solver.e);
  const SolverOptions& o = solver_options();  // EPSSetFromOptions
  if (rc == ED_OK && (o.eps_tol > 0.0 || o.eps_max_it > 0)) rc = ed_eps_set_tolerances(solver.e, o.eps_tol, o.eps_max_it);
  return rc;
}
inline PetscErrorCode EPSSetDimensions(EPS& solver, PetscInt nev, PetscInt ncv, PetscInt mpd) {
  return ed_eps_set_dimensions(solver.e, (int)nev, (int)ncv, (int)mpd);
}
inline PetscErrorCode EPSSetTolerances(EPS& solver, PetscReal tol, PetscInt max_it) {
  return ed_eps_set_tolerances(solver.e, tol, (int)max_it);
}
inline PetscErrorCode solve(Environment&, EPS& solver, PetscInt& nconv) {
  int n = 0;
  int rc = ed_eps_solve(solver.e, &n);
  nconv = n;
  return rc;
}
// Solver::solution (src/solver.cpp:58-68): eigenvalue, relative error, and
// the eigenvector copied into the device vector x (from MatCreateVecs).
inline PetscErrorCode solution(EPS& solver, PetscInt index, PetscScalar& value, Vec& x, PetscReal& error) {
  double ev = 0.0, err = 0.0;
  int rc = ed_eps_get_eigenpair(solver.e, (int)index, &ev, &err, x ? x->d : nullptr);
  value = PetscScalar(ev, 0.0);
  error = err;
  return rc;
}
// The same with the eigenvalue in a double (drivers written for a real PETSc
// build, e.g. examples/ex1.cpp).
inline PetscErrorCode solution(EPS& solver, PetscInt index, double& value, Vec& x, double& error) {
  PetscScalar v;
  int rc = solution(solver, index, v, x, error);
  value = v.re;
  return rc;
}
inline PetscErrorCode SolverClean(EPS& solver) {
  int rc = ed_eps_destroy(solver.e);
  solver.e = nullptr;
  return rc;
}
}  // namespace Solver

// ---------------------------------------------------------------------------
// Correlations (include/spinOperators/correlation.hpp:80-194)
// ---------------------------------------------------------------------------
class Correlation {
 protected:
  Basis& basis;
  int op;
  Correlation(Basis& b, int o) : basis(b), op(o) {}
 public:
  PetscScalar ExpectVal(Environment&, PetscInt spin_i, PetscInt spin_j, Vec& state) {
    int32_t pr[2] = {(int32_t)spin_i, (int32_t)spin_j};
    ed_cplx out;
    throw_on(ed_expect_pairs(basis.h, op, state->d, pr, 1, &out));
    return PetscScalar(out.re, out.im);
  }
  // All N*N values in one fused pass (row-major [i][j]).
  std::vector<PetscScalar> AllPairs(Vec& state) {
    std::vector<PetscScalar> out((size_t)(basis.nspins * basis.nspins));
    std::vector<ed_cplx> tmp(out.size());
    throw_on(ed_expect_all_pairs(basis.h, op, state->d, tmp.data()));
    for (size_t k = 0; k < tmp.size(); ++k) out[k] = PetscScalar(tmp[k].re, tmp[k].im);
    return out;
  }
};
class SzSz : public Correlation { public: SzSz(Environment&, Basis& b) : Correlation(b, ED_OP_SZSZ) {} };
class SpSm : public Correlation { public: SpSm(Environment&, Basis& b) : Correlation(b, ED_OP_SPSM) {} };
class SmSp : public Correlation { public: SmSp(Environment&, Basis& b) : Correlation(b, ED_OP_SMSP) {} };
class SiSj : public Correlation { public: SiSj(Environment&, Basis& b) : Correlation(b, ED_OP_SISJ) {} };

// ---------------------------------------------------------------------------
// Sublattices (src/sublattice.cpp:5-91) and order parameters
// (include/phys.tmpl_func.hpp:5-81)
// ---------------------------------------------------------------------------
template <typename L>
class AF {
 public:
  std::vector<std::vector<PetscInt>> sublat{{}, {}};
  AF(L& lat, PetscInt /*size*/ = 2) {
    if (lat.nspins_x == 1) {
      for (PetscInt i = 0; i < lat.nspins; ++i) sublat[(i % 2) ? 1 : 0].push_back(i);
    } else {
      int tagx = 0;
      for (PetscInt ix = 0; ix < lat.nspins_x; ++ix) {
        int tagy = tagx;
        for (PetscInt iy = 0; iy < lat.nspins_y; ++iy) {
          sublat[(tagy % 2) ? 1 : 0].push_back(ix * lat.nspins_y + iy);
          tagy ^= 1;
        }
        tagx ^= 1;
      }
    }
  }
  PetscInt get_size() const { return 2; }
  const std::vector<PetscInt>& get_sl(PetscInt i) const { return sublat[(size_t)i]; }
};

template <typename L>
class Striped {
 public:
  std::vector<std::vector<PetscInt>> sublat{{}, {}, {}, {}};
  Striped(L& lat, PetscInt /*size*/ = 4) {
    int tagx = 0;
    for (PetscInt ix = 0; ix < lat.nspins_x; ++ix) {
      int tagy = 0;
      for (PetscInt iy = 0; iy < lat.nspins_y; ++iy) {
        PetscInt cur = ix * lat.nspins_y + iy;
        sublat[(tagy % 2) ? 1 : 0].push_back(cur);
        sublat[(tagx % 2) ? 3 : 2].push_back(cur);
        tagy ^= 1;
      }
      tagx ^= 1;
    }
  }
  PetscInt get_size() const { return 4; }
  const std::vector<PetscInt>& get_sl(PetscInt i) const { return sublat[(size_t)i]; }
};

namespace Phys {
inline PetscScalar sublattice_sum(Basis& b, const std::vector<const std::vector<PetscInt>*>& lists, Vec& state) {
  std::vector<int32_t> pairs;
  for (auto* sl : lists)
    for (PetscInt i : *sl)
      for (PetscInt j : *sl) { pairs.push_back((int32_t)i); pairs.push_back((int32_t)j); }
  std::vector<ed_cplx> out(pairs.size() / 2);
  throw_on(ed_expect_pairs(b.h, ED_OP_SISJ, state->d, pairs.data(), (int64_t)out.size(), out.data()));
  PetscScalar e = 0.0;
  for (auto& v : out) e += PetscScalar(v.re, v.im);
  return e;
}
template <typename L>
inline PetscScalar SquaredSubLattMagAF(Environment& env, Basis& b, AF<L>& sl, Vec& state) {
  PetscScalar e = sublattice_sum(b, {&sl.get_sl(0), &sl.get_sl(1)}, state);
  return e * 8.0 / PetscScalar((double)env.nspins) / PetscScalar(env.nspins + 4.0);
}
template <typename L>
inline PetscScalar SquaredSubLattMagSTR(Environment& env, Basis& b, Striped<L>& sl, Vec& state) {
  PetscScalar e = sublattice_sum(b, {&sl.get_sl(0), &sl.get_sl(1), &sl.get_sl(2), &sl.get_sl(3)}, state);
  return e * 4.0 / PetscScalar((double)env.nspins) / PetscScalar(env.nspins + 4.0);
}

// DSF_data (include/phys.hpp:25-39): the same fields.
template <typename L>
struct DSF_data {
  DSF_data() {}
  Basis* b0 = nullptr;            // basis of the state's sector
  Basis* b1 = nullptr;            // basis of the sector SQ maps to (b0 for Sqz)
  L* lat = nullptr;
  Hamiltonian<L>* h0 = nullptr;   // its couplings go to the file header
  Hamiltonian<L>* h1 = nullptr;   // solved for nev eigenpairs
  PetscInt nev = 10, ncv = PETSC_DEFAULT, mpd = PETSC_DEFAULT;
  bool disorder = false;
  PetscReal* hi = nullptr;        // nspins fields, written to the header when disorder
  const char* path = "./";
};
}  // namespace Phys

// Operator tags of DynStructFactor: S^z_i within the sector
// (spinOPft.tmpl_func.hpp:28-60) and S^+_i from sector m to m+1
// (spinOPft.tmpl_func.hpp:77-143).
struct Sqz { static constexpr int op = 0; };
struct Sqp { static constexpr int op = 1; };

namespace Phys {
// DynStructFactor<L, SQ> (include/phys.tmpl_func.hpp:87-215): nev lowest
// eigenpairs of h1 (SLEPc's default tolerance, as the reference sets none),
// c_{i,n} = <n| SQ_i |state> for every site, and the file
// <path>/dsf_d<dis_iter>.dat in the reference's layout.
template <typename L, typename SQ>
inline PetscErrorCode DynStructFactor(Environment& env, DSF_data<L>& data, PetscScalar gs, Vec& state,
                                      PetscInt dis_iter = 0) {
  EPS solver;
  PetscErrorCode rc = Solver::SolverInit(solver, data.h1->hamilt, data.nev, data.ncv, data.mpd);
  if (rc != ED_OK) return rc;
  PetscInt nconv = 0;
  const int nev = (int)data.nev;
  const size_t dim1 = (size_t)data.b1->size;
  Vec vecs = nullptr;
  rc = VecCreateOnDevice(env.ctx, (PetscInt)(dim1 * (size_t)nev), &vecs);
  if (rc != ED_OK) {
    Solver::SolverClean(solver);
    return rc;
  }
  std::vector<double> ev((size_t)nev);
  rc = Solver::solve(env, solver, nconv);
  for (int n = 0; n < nev && rc == ED_OK; ++n) {
    double er = 0.0;
    rc = ed_eps_get_eigenpair(solver.e, n, &ev[(size_t)n], &er, vecs->d + (size_t)n * dim1);
  }
  std::vector<ed_cplx> c((size_t)env.nspins * (size_t)nev);
  if (rc == ED_OK) rc = ed_dsf_coefficients(data.b0->h, data.b1->h, SQ::op, state->d, vecs->d, nev, c.data());
  Solver::SolverClean(solver);
  VecDestroy(&vecs);
  if (rc != ED_OK) return rc;
  const std::string fn = std::string(data.path) + "/dsf_d" + std::to_string((long)dis_iter) + ".dat";
  FILE* fp = std::fopen(fn.c_str(), "w");
  if (!fp) throw std::runtime_error("Cannot open file");
  std::fprintf(fp, "#------------------------------- Parameters -------------------------------------\n");
  std::fprintf(fp, "#%7s:   %ld  \n", " nspins", (long)env.nspins);
  std::fprintf(fp, "#%7s:   %ld  \n", " nev", (long)data.nev);
  std::fprintf(fp, "#%7s:   %.16f  \n", " GS", gs.re);
  std::fprintf(fp, "#%7s:   %.5f  %4s:   %.5f  %4s:   %.5f  %4s:   %.5f\n", "J1", data.h0->hamilt_J1(), "D1",
               data.h0->hamilt_D1(), "J2", data.h0->hamilt_J2(), "D2", data.h0->hamilt_D2());
  if (data.disorder)
    for (PetscInt i = 0; i < env.nspins; ++i) std::fprintf(fp, "# hi[%4ld]: %.16f\n", (long)i, data.hi[i]);
  std::fprintf(fp, "#--------------------------------------------------------------------------------\n#\n#\n");
  std::fprintf(fp, "#----- Energy -----  ------ Factor -----\n");
  for (PetscInt s = 0; s < env.nspins; ++s) {
    std::fprintf(fp, "# spin: %ld\n", (long)s);
    for (int n = 0; n < nev; ++n)
      std::fprintf(fp, "%.13e  %.13e\n", ev[(size_t)n] - gs.re, c[(size_t)s * (size_t)nev + (size_t)n].re);
  }
  std::fclose(fp);
  return ED_OK;
}
}  // namespace Phys

}  // namespace lsqed
