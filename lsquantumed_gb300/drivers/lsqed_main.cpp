// lsqed_main — drop-in for the reference drivers examples/main.cpp and
// examples/main_disorder.cpp on one GPU, written against the lsqed.hpp shim.
//
// Flags (include/tools/parse_args.hpp:34-66; names are matched without case
// like the PETSc options database):
//   -n <N> -ltype chain1D|square2D|honeycomb2D -lx <lx> -ly <ly>
//   -j1 <J1> -d1 <D1> -j2 <J2> -d2 <D2>
//   -disorder [-min_dis a -max_dis b -rep k -reprod 0|1]
//   -eps_type krylovschur -eps_tol <tol> -eps_nev <nev> -eps_ncv <ncv> -eps_max_it <it>
//   -dsf_nev <nev>  (DynStructFactor; 0 skips it)   -path <dir>
// -nn / -nnn of the legacy parser are accepted and ignored.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lsqed/lsqed.hpp"

using namespace lsqed;

static std::string lower(std::string s) {
  std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
  return s;
}

struct Args {
  PetscInt n = 6, lx = 1, ly = -1;
  std::string ltype = "chain1d";
  double J1 = 1.0, D1 = 1.0, J2 = 0.0, D2 = 0.0;
  bool disorder = false, reprod = true;
  double min_dis = -0.3, max_dis = 0.3;
  PetscInt rep = 1;
  double tol = 1e-8;
  int nev = 1, ncv = -1, max_it = 0, dsf_nev = 10;
  std::string path = "./";
};

static Args parse(int argc, char** argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    std::string k = lower(argv[i]);
    auto val = [&](const char* what) -> std::string {
      if (i + 1 >= argc) throw std::invalid_argument(std::string("missing value for ") + what);
      return argv[++i];
    };
    if (k == "-n") a.n = std::atol(val("-n").c_str());
    else if (k == "-ltype") a.ltype = lower(val("-ltype"));
    else if (k == "-lx") a.lx = std::atol(val("-lx").c_str());
    else if (k == "-ly") a.ly = std::atol(val("-ly").c_str());
    else if (k == "-j1") a.J1 = std::atof(val("-j1").c_str());
    else if (k == "-d1") a.D1 = std::atof(val("-d1").c_str());
    else if (k == "-j2") a.J2 = std::atof(val("-j2").c_str());
    else if (k == "-d2") a.D2 = std::atof(val("-d2").c_str());
    else if (k == "-disorder") a.disorder = true;
    else if (k == "-min_dis") a.min_dis = std::atof(val("-min_dis").c_str());
    else if (k == "-max_dis") a.max_dis = std::atof(val("-max_dis").c_str());
    else if (k == "-rep") a.rep = std::atol(val("-rep").c_str());
    else if (k == "-reprod") a.reprod = std::atoi(val("-reprod").c_str()) != 0;
    else if (k == "-eps_tol") a.tol = std::atof(val("-eps_tol").c_str());
    else if (k == "-eps_nev") a.nev = std::atoi(val("-eps_nev").c_str());
    else if (k == "-eps_ncv") a.ncv = std::atoi(val("-eps_ncv").c_str());
    else if (k == "-eps_max_it") a.max_it = std::atoi(val("-eps_max_it").c_str());
    else if (k == "-eps_type") {
      std::string t = lower(val("-eps_type"));
      if (t != "krylovschur") throw std::invalid_argument("only -eps_type krylovschur is provided");
    } else if (k == "-dsf_nev") a.dsf_nev = std::atoi(val("-dsf_nev").c_str());
    else if (k == "-path") a.path = val("-path");
    else if (k == "-nn" || k == "-nnn") continue;  // legacy flags (parse_args.hpp.old), ignored by the reference too
    else std::fprintf(stderr, "warning: unused option %s\n", argv[i]);
  }
  if (a.n % 2 != 0) throw std::invalid_argument("The total number of spins has to be EVEN.");
  if (a.n <= 0) throw std::invalid_argument("The total number of spins has to be POSITIVE.");
  if (a.ly < 0) a.ly = a.n;
  if (!a.disorder) { a.min_dis = 0.0; a.max_dis = 0.0; a.reprod = true; a.rep = 1; }
  return a;
}

template <typename L>
static int run(Environment& env, L& lat, const Args& a) {
  Basis b{env, 0};
  Hamiltonian<L> h{env, b, lat, a.J1, a.D1, a.J2, a.D2};
  h.build_diag(env);
  h.build_off_diag(env);
  std::vector<int64_t> seeds((size_t)a.rep);
  throw_on(ed_random_seeds(a.reprod ? 1 : 0, a.rep, seeds.data()));
  std::vector<double> hi((size_t)a.n, 0.0);
  Vec state = nullptr;
  throw_on(MatCreateVecs(h.hamilt, &state, nullptr));
  double magAF = 0.0, magSTR = 0.0;
  std::printf(" iter          k          ||Ax-kx||/||kx||\n ----    -------------   ------------------\n");
  for (PetscInt repet = 0; repet < a.rep; ++repet) {
    if (a.disorder) {
      throw_on(ed_random_fields(seeds[(size_t)repet], (int)a.n, a.min_dis, a.max_dis, hi.data()));
      throw_on(h.build_disorder(env, hi.data()));
    }
    EPS solver;
    throw_on(Solver::SolverInit(solver, h.hamilt, a.nev, a.ncv));
    throw_on(Solver::EPSSetTolerances(solver, a.tol, a.max_it));
    PetscInt nconv = 0;
    throw_on(Solver::solve(env, solver, nconv));
    PetscScalar eig;
    PetscReal err;
    if (nconv > 0) {
      throw_on(Solver::solution(solver, 0, eig, state, err));
      std::printf("  %ld     %12f       %12g\n\n", (long)repet, PetscRealPart(eig), err);
    }
    Solver::SolverClean(solver);
    AF<L> af{lat, 2};
    magAF += Phys::SquaredSubLattMagAF(env, b, af, state).real();
    std::printf("magAF: %.10f\n", magAF / (double)a.rep);
    if (lat.nspins_x > 1 && a.ltype == "square2d") {
      Striped<L> st{lat, 4};
      magSTR += Phys::SquaredSubLattMagSTR(env, b, st, state).real();
      std::printf("magSTR: %.10f\n", magSTR / (double)a.rep);
    }
    if (a.dsf_nev > 0) {
      // examples/main.cpp:89-98: the DSF of the ground state within the sector
      Phys::DSF_data<L> dsf_data;
      dsf_data.b0 = &b;
      dsf_data.b1 = &b;
      dsf_data.lat = &lat;
      dsf_data.h0 = &h;
      dsf_data.h1 = &h;
      dsf_data.nev = a.dsf_nev;
      dsf_data.ncv = PETSC_DECIDE;
      dsf_data.mpd = PETSC_DECIDE;
      dsf_data.disorder = a.disorder;
      dsf_data.hi = a.disorder ? hi.data() : nullptr;
      dsf_data.path = a.path.c_str();
      throw_on(Phys::DynStructFactor<L, Sqz>(env, dsf_data, eig, state, repet));
    }
  }
  VecDestroy(&state);
  return 0;
}

int main(int argc, char** argv) {
  try {
    Args a = parse(argc, argv);
    Environment env{argc, argv, a.n};
    env.disorder_flg = a.disorder;
    std::printf(" ------ Parameters ------\n%9s:   %ld\n", "spins", (long)a.n);
    std::printf("%9s:   %.5f\n%9s:   %.5f\n%9s:   %.5f\n%9s:   %.5f\n", "J1", a.J1, "D1", a.D1, "J2", a.J2, "D2", a.D2);
    std::printf(" ------------------------\n%9s:   %4s\n ------------------------\n\n", "disorder",
                a.disorder ? "TRUE" : "FALSE");
    if (a.ltype == "chain1d") {
      chain1D lat{env};
      return run(env, lat, a);
    } else if (a.ltype == "square2d") {
      square2D lat{env, a.lx, a.ly};
      return run(env, lat, a);
    } else if (a.ltype == "honeycomb2d") {
      honeycomb2D lat{env, a.lx, a.ly};
      return run(env, lat, a);
    }
    throw std::invalid_argument("unknown -ltype " + a.ltype);
  } catch (const std::exception& ex) {
    std::fprintf(stderr, "error: %s\n", ex.what());
    return 1;
  }
}
