// lsqed_dropin.hpp — one header that stands in for every header a driver of
// the reference includes (sublattice.hpp, time_monitor.hpp,
// random_disorder.hpp, parse_args.hpp, print_args.hpp, phys.hpp,
// hamiltonian.hpp, solver.hpp, petsctime.h ...): the lsqed.hpp classes in the
// global namespace, plus what those drivers call from PETSc and from the
// reference's tools:
//   * PetscPrintf, CHKERRQ, PETSC_COMM_WORLD / MPI_COMM_WORLD (one process);
//   * PetscLogStage*, MatAssemblyBegin/End, MatGetInfo (no-ops or what the
//     matrix-free operator can report: the matrix is never assembled);
//   * TIME_IT as the reference defines it without TIME_CODE;
//   * parse_args() / print_args(): the reference's macros
//     (include/tools/parse_args.hpp:13-76, print_args.hpp:12-39), the same
//     local variables, defaults, checks and option names, read from the
//     command line that Environment saw;
//   * Tools::RandomDisorder (include/tools/random_disorder.hpp), on the C
//     ABI's libstdc++ draws.
// Drivers of the reference compile with their #include lines replaced by
// this one (checked by tests/test_shim_dropin_cpu.py).
#pragma once
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "lsqed.hpp"

using namespace lsqed;

// ---- communicators, printing, error checks ---------------------------------
typedef int MPI_Comm;
static const MPI_Comm PETSC_COMM_WORLD = 0;
static const MPI_Comm MPI_COMM_WORLD = 0;
typedef int PetscMPIInt;

namespace lsqed {
// complex scalars print as their real part (PETSc's %f on a complex scalar)
inline double print_arg(const Scalar& z) { return z.re; }
inline int print_arg(PetscBool b) { return (int)b; }
template <typename T>
inline T print_arg(T v) { return v; }
}  // namespace lsqed

template <typename... A>
inline PetscErrorCode PetscPrintf(MPI_Comm, const char* fmt, A... args) {
  std::printf(fmt, lsqed::print_arg(args)...);
  return 0;
}
inline PetscErrorCode PetscPrintf(MPI_Comm, const char* fmt) {
  std::fputs(fmt, stdout);
  return 0;
}

#define CHKERRQ(ierr)                 \
  do {                                \
    if ((ierr) != 0) return (ierr);   \
  } while (0)

// ---- logging stages and matrix assembly ------------------------------------
typedef int PetscLogStage;
inline PetscErrorCode PetscLogStageRegister(const char*, PetscLogStage* s) {
  static int next = 0;
  *s = next++;
  return 0;
}
inline PetscErrorCode PetscLogStagePush(PetscLogStage) { return 0; }
inline PetscErrorCode PetscLogStagePop() { return 0; }

enum MatAssemblyType { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 };
enum MatInfoType { MAT_LOCAL = 1, MAT_GLOBAL_MAX = 2, MAT_GLOBAL_SUM = 3 };
struct MatInfo {
  double block_size, nz_allocated, nz_used, nz_unneeded, memory, assemblies, mallocs, fill_ratio_given,
      fill_ratio_needed, factor_mallocs;
};
// The operator is matrix-free on the device: nothing to assemble.
inline PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
inline PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType) { return 0; }
// No stored entries, one "assembly" (build_diag / build_off_diag).
inline PetscErrorCode MatGetInfo(Mat A, MatInfoType, MatInfo* info) {
  if (!A || !info) return 1;
  std::memset(info, 0, sizeof(MatInfo));
  info->block_size = 1;
  info->assemblies = 1;
  return 0;
}

// ---- timing (include/tools/time_monitor.hpp:31-33 without TIME_CODE) --------
#define TIME_IT(tm, func_name, func) (func);

// ---- lattice type and option parsing ----------------------------------------
enum class lattice_type { chain1D, square2D, honeycomb2D };

namespace lsqed {
// Value of option `name` (case-insensitive, as PETSc matches options) from
// the command line Environment saw; nullptr when absent.  `flag` options
// (no value) report "" when present.
inline const char* option_value(const char* name, bool flag = false) {
  const std::vector<std::string>& a = command_line().args;
  auto eq = [](const std::string& x, const char* y) {
    if (x.size() != std::strlen(y)) return false;
    for (size_t k = 0; k < x.size(); ++k)
      if (std::tolower((unsigned char)x[k]) != std::tolower((unsigned char)y[k])) return false;
    return true;
  };
  for (size_t k = 1; k < a.size(); ++k)
    if (eq(a[k], name)) {
      if (flag) return "";
      return k + 1 < a.size() ? a[k + 1].c_str() : nullptr;
    }
  return nullptr;
}
inline void option_int(const char* name, PetscInt& v) {
  if (const char* s = option_value(name)) v = (PetscInt)std::atol(s);
}
inline void option_real(const char* name, PetscReal& v) {
  if (const char* s = option_value(name)) v = std::atof(s);
}
inline void option_bool(const char* name, PetscBool& v) {
  if (const char* s = option_value(name, true)) {
    const char* val = option_value(name);
    // "-reprod" alone, or followed by another option, means true
    if (!val || val[0] == '-' || !std::strlen(val)) v = PETSC_TRUE;
    else v = (std::strcmp(val, "0") && std::strcmp(val, "false") && std::strcmp(val, "FALSE")) ? PETSC_TRUE
                                                                                             : PETSC_FALSE;
    (void)s;
  }
}
inline bool option_present(const char* name) { return option_value(name, true) != nullptr; }
inline void option_lattice(lattice_type& t, PetscBool& found) {
  const char* s = option_value("-ltype");
  if (!s) return;
  found = PETSC_TRUE;
  std::string v = s;
  if (v == "chain1D") t = lattice_type::chain1D;
  else if (v == "square2D") t = lattice_type::square2D;
  else if (v == "honeycomb2D") t = lattice_type::honeycomb2D;
  else throw std::invalid_argument("Unknown lattice type " + v);
}
}  // namespace lsqed

// parse_args() (include/tools/parse_args.hpp:13-76): declares the driver's
// parameters with the reference's defaults and fills them from -n, -ltype,
// -lx, -ly, -j1, -d1, -j2, -d2, -disorder (-min_dis, -max_dis, -rep,
// -reprod); -lx / -ly are rejected for chain1D; an odd or non-positive
// number of spins throws std::invalid_argument.  Uses `env` like the
// reference's macro.
#define parse_args()                                                                                    \
  PetscInt _n = (env.nspins == 0) ? 6 : env.nspins;                                                     \
  lsqed::option_int("-n", _n);                                                                          \
  PetscInt lx = 1;                                                                                      \
  PetscInt ly = _n;                                                                                     \
  PetscReal J1 = 1.0;                                                                                   \
  PetscReal Delta1 = 1.0;                                                                               \
  PetscReal J2 = 0.0;                                                                                   \
  PetscReal Delta2 = 0.0;                                                                               \
  PetscInt rep = 1;                                                                                     \
  PetscReal min_dis = -0.3;                                                                             \
  PetscReal max_dis = 0.3;                                                                              \
  PetscBool reprod = PETSC_TRUE;                                                                        \
  PetscBool check_dis = PETSC_FALSE;                                                                    \
  PetscBool check_lattype = PETSC_FALSE;                                                                \
  lattice_type ltype = lattice_type::chain1D;                                                           \
  if (_n % 2 != 0) throw std::invalid_argument("The total number of spins has to be EVEN.");            \
  if (_n <= 0) throw std::invalid_argument("The total number of spins has to be POSITIVE.");           \
  env.nspins = _n;                                                                                      \
  lsqed::option_lattice(ltype, check_lattype);                                                          \
  if (ltype == lattice_type::chain1D) {                                                                 \
    if (lsqed::option_present("-lx") || lsqed::option_present("-ly"))                                   \
      throw std::invalid_argument(                                                                      \
          "For chain1D lattice, one should not specify the dimension in each direction");              \
  } else {                                                                                              \
    lsqed::option_int("-lx", lx);                                                                       \
    lsqed::option_int("-ly", ly);                                                                       \
  }                                                                                                     \
  lsqed::option_real("-j1", J1);                                                                        \
  lsqed::option_real("-d1", Delta1);                                                                    \
  lsqed::option_real("-j2", J2);                                                                        \
  lsqed::option_real("-d2", Delta2);                                                                    \
  if (lsqed::option_present("-disorder")) check_dis = PETSC_TRUE;                                       \
  if (check_dis) {                                                                                      \
    env.disorder_flg = true;                                                                            \
    lsqed::option_real("-min_dis", min_dis);                                                            \
    lsqed::option_real("-max_dis", max_dis);                                                            \
    lsqed::option_int("-rep", rep);                                                                     \
    lsqed::option_bool("-reprod", reprod);                                                              \
  }                                                                                                     \
  check_lattype = PETSC_TRUE;                                                                           \
  if (env.disorder_flg == false) {                                                                      \
    max_dis = 0.0;                                                                                      \
    min_dis = 0.0;                                                                                      \
    reprod = PETSC_TRUE;                                                                                \
    rep = 1;                                                                                            \
  }

// print_args() (include/tools/print_args.hpp:12-39): the parameter block.
#define print_args()                                                                                    \
  ierr = PetscPrintf(PETSC_COMM_WORLD, " ------ Parameters ------\n"); CHKERRQ(ierr);                   \
  ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %d\n", "spins", (int)env.nspins); CHKERRQ(ierr);         \
  if (check_lattype == true) {                                                                          \
    switch (ltype) {                                                                                    \
      case lattice_type::chain1D: {                                                                     \
        ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %7s\n", "lattice", "chain1D"); CHKERRQ(ierr);      \
        break;                                                                                          \
      }                                                                                                 \
      case lattice_type::square2D: {                                                                    \
        ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %8s\n", "lattice", "square2D"); CHKERRQ(ierr);     \
        ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %d\n%9s:   %d\n", "Lx", (int)lx, "Ly", (int)ly);   \
        CHKERRQ(ierr);                                                                                  \
        break;                                                                                          \
      }                                                                                                 \
      case lattice_type::honeycomb2D: {                                                                 \
        ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %10s\n", "lattice", "honeycomb2D"); CHKERRQ(ierr); \
        break;                                                                                          \
      }                                                                                                 \
    }                                                                                                   \
  }                                                                                                     \
  ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %.5f\n%9s:   %.5f\n", "J1", J1, "D1", Delta1);          \
  CHKERRQ(ierr);                                                                                        \
  ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %.5f\n%9s:   %.5f\n", "J2", J2, "D2", Delta2);          \
  CHKERRQ(ierr);                                                                                        \
  if (check_dis == true) {                                                                              \
    ierr = PetscPrintf(PETSC_COMM_WORLD, " ------------------------\n"); CHKERRQ(ierr);                 \
    ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %4s\n", "disorder", "TRUE"); CHKERRQ(ierr);            \
    ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %.5f\n%9s:   %.5f\n", "min dis", min_dis, "max dis",   \
                       max_dis);                                                                        \
    CHKERRQ(ierr);                                                                                      \
    ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %d\n%9s:   %d\n", "reprod?", (int)reprod, "rep",       \
                       (int)rep);                                                                       \
    CHKERRQ(ierr);                                                                                      \
  } else {                                                                                              \
    ierr = PetscPrintf(PETSC_COMM_WORLD, " ------------------------\n"); CHKERRQ(ierr);                 \
    ierr = PetscPrintf(PETSC_COMM_WORLD, "%9s:   %4s\n", "disorder", "FALSE"); CHKERRQ(ierr);           \
  }                                                                                                     \
  ierr = PetscPrintf(PETSC_COMM_WORLD, " ------------------------\n\n"); CHKERRQ(ierr);

// ---- Tools::RandomDisorder (src/tools/random_disorder.cpp:33-59) -----------
namespace Tools {
class RandomDisorder {
 public:
  PetscReal* hi = nullptr;
  PetscInt* srand_seq = nullptr;
  PetscInt nspins = 0, rep = 0;
  PetscReal min = 0.0, max = 0.0;
  RandomDisorder() {}
  RandomDisorder(PetscInt m_nspins, PetscBool m_reprod, PetscReal m_min, PetscReal m_max, PetscInt m_rep)
      : nspins(m_nspins), rep(m_rep), min(m_min), max(m_max) {
    hi = new PetscReal[(size_t)nspins];
    srand_seq = srand_seq_init(m_reprod);
  }
  ~RandomDisorder() {
    delete[] hi;
    delete[] srand_seq;
  }
  RandomDisorder(const RandomDisorder&) = delete;
  RandomDisorder& operator=(const RandomDisorder&) = delete;
  // rep seeds from mt19937_64(1) when reproducible, else std::random_device
  PetscInt* srand_seq_init(PetscBool reprod) {
    PetscInt* s = new PetscInt[(size_t)(rep > 0 ? rep : 1)];
    lsqed::throw_on(ed_random_seeds(reprod ? 1 : 0, rep, reinterpret_cast<int64_t*>(s)));
    return s;
  }
  // h_i ~ uniform_real(min, max) from mt19937_64(srand_seq[dis_index])
  void hi_init(PetscInt dis_index) {
    lsqed::throw_on(ed_random_fields(srand_seq[dis_index], (int)nspins, min, max, hi));
  }
};
}  // namespace Tools
