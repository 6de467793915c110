// Compile-only check of the lsqed.hpp shim (tests/test_capi_cpu.py): every
// class and template of the reference's interface instantiated once for each
// lattice, as a driver written against the reference would use them.
#include "lsqed/lsqed.hpp"
using namespace lsqed;

template <typename L>
void use_all(Environment& env, L& lat) {
  Basis b0{env, 0}, b1{env, 1};
  Hamiltonian<L> h0{env, b0, lat, 1.0, 1.0, 0.5, 0.5}, h1{env, b1, lat, 1.0, 1.0, 0.5, 0.5};
  h0.build_diag(env);
  h0.build_off_diag(env);
  Vec state = nullptr;
  MatCreateVecs(h0.hamilt, &state, nullptr);
  EPS eps;
  Solver::SolverInit(eps, h0.hamilt, 2);
  Solver::EPSSetTolerances(eps, 1e-9, 0);
  PetscInt nconv = 0;
  Solver::solve(env, eps, nconv);
  PetscScalar e0;
  PetscReal err;
  Solver::solution(eps, 0, e0, state, err);
  Solver::SolverClean(eps);
  SiSj sisj{env, b0};
  SzSz szsz{env, b0};
  SpSm spsm{env, b0};
  SmSp smsp{env, b0};
  sisj.ExpectVal(env, 0, 1, state);
  szsz.ExpectVal(env, 0, 1, state);
  spsm.ExpectVal(env, 0, 1, state);
  smsp.ExpectVal(env, 0, 1, state);
  AF<L> af{lat, 2};
  Phys::SquaredSubLattMagAF(env, b0, af, state);
  Phys::DSF_data<L> d;
  d.b0 = &b0;
  d.b1 = &b1;
  d.lat = &lat;
  d.h0 = &h0;
  d.h1 = &h1;
  Phys::DynStructFactor<L, Sqp>(env, d, e0, state, 1);
  d.b1 = &b0;
  d.h1 = &h0;
  Phys::DynStructFactor<L, Sqz>(env, d, e0, state);
  double e1 = 0.0, err1 = 0.0;
  Solver::solution(eps, 0, e1, state, err1);
  double m2 = Phys::SquaredSubLattMagAF(env, b0, af, state);
  (void)m2;
  VecDestroy(&state);
}

int main(int argc, char** argv) {
  Environment env{argc, argv, 16};
  chain1D chain{env};
  square2D square{env, 4, 4};
  honeycomb2D honey{env, 2, 4};
  use_all(env, chain);
  use_all(env, square);
  use_all(env, honey);
  Striped<square2D> st{square, 4};
  Basis b{env, 0};
  Vec v = nullptr;
  VecCreateOnDevice(env.ctx, b.size, &v);
  Phys::SquaredSubLattMagSTR(env, b, st, v);
  VecDestroy(&v);
  return 0;
}
