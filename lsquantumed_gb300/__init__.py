"""GB300-native exact diagonalization of spin-1/2 J1-J2 Heisenberg models.

The compute path is libedgb300.so (hand-written sm_103a CUDA kernels behind
the C ABI in include/ed_capi.h); this package is the host-side mirror of the
LSQuantumED interfaces (Basis, Hamiltonian, Solver, SiSj, Phys, ...).
"""
from . import capi  # noqa: F401
from .capi import EDError, InvalidArgument  # noqa: F401
from .ed import (AF, Adjoint, DSF_data, EPS, DisorderBatch, PETSC_DECIDE, PETSC_DEFAULT, Basis, Environment, Hamiltonian,  # noqa: F401
                 Phys, RandomDisorder, SiSj, SmSp, Solver, SpSm, Striped, SzSz, chain1D, honeycomb2D,
                 bv_dot_real, bv_mult_real, ground_state_energy, random_fields, random_normal, solve_batches,
                 square2D)


def build(force=False):
    from .build import build as _b
    return _b(force=force)
