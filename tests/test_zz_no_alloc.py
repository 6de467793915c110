"""ed_ham_apply_noalloc: the H.v entry point for callers that cannot let a
library allocate device memory (a framework that owns the device memory pool,
or a loop that cannot afford an allocation's synchronisation).  It keeps its
scratch in one static device array, so the call allocates nothing.

Checked through the C ABI against ed_ham_apply, which computes the same
fixed-point H.v with buffers it allocates itself, and against the oracle's
explicit-matrix product: two calls in a row (the shared scratch must not
carry stale state into the second call), within the H.v tolerance the other
tests use (1e-14 * ||x||_2).  This file is collected last so a failure here
leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def setup():
    from lsquantumed_gb300.build import build
    build()
    import lsquantumed_gb300 as ed
    return ed


def _ham(ed, env, N, lx, ly, mag):
    b = ed.Basis(env, mag)
    lat = ed.square2D(env, lx, ly)
    h = ed.Hamiltonian(env, b, lat, 1.0, 1.0, 0.5, 0.5)
    h.build_diag(env)
    h.build_off_diag(env)
    return b, h


def test_noalloc_matches_apply_twice(setup):
    import torch
    import oracle
    ed = setup
    lib = ed.capi.lib()
    env = ed.Environment(nspins=20)
    b, h = _ham(ed, env, 20, 4, 5, 0)
    h.set_accumulation('fixed64')
    M = oracle.Model(1, 20, 4, 5, 0, 1.0, 1.0, 0.5, 0.5)
    M.build(3)
    gen = torch.Generator(device='cuda').manual_seed(1234)
    for call in range(2):
        x = torch.complex(torch.rand(b.size, dtype=torch.float64, device='cuda', generator=gen) * 2 - 1,
                          torch.rand(b.size, dtype=torch.float64, device='cuda', generator=gen) * 2 - 1)
        if call == 1:
            x = x * 1e-3  # different scale: the shared exponent must be recomputed, not reused
        y_ref = torch.empty_like(x)
        y_new = torch.full_like(x, float('nan'))
        assert lib.ed_ham_apply(h.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_ref.data_ptr())) == 0
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = lib.ed_ham_apply_noalloc(h.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_new.data_ptr()))
        assert rc == 0, ed.capi.last_error()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:  # the first call may finish loading the module; later calls must not allocate
            assert free_after >= free_before
        tol = 1e-14 * torch.linalg.vector_norm(x).item()
        err = (y_new - y_ref).abs().max().item()
        assert err <= tol, (call, err, tol)
        err_orc = np.abs(y_new.cpu().numpy() - M.apply(x.cpu().numpy())).max()
        assert err_orc <= tol, (call, err_orc, tol)


def test_noalloc_rejects_large_basis(setup):
    ed = setup
    lib = ed.capi.lib()
    env = ed.Environment(nspins=26)
    b = ed.Basis(env, 0)  # C(26,13) = 10,400,600 states > 2^22
    lat = ed.chain1D(env)
    h = ed.Hamiltonian(env, b, lat, 1.0, 1.0, 0.0, 0.0)
    h.build_diag(env)
    h.build_off_diag(env)
    import torch
    x = torch.zeros(b.size, dtype=torch.complex128, device='cuda')
    y = torch.zeros_like(x)
    rc = lib.ed_ham_apply_noalloc(h.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()))
    assert rc == ed.capi.ED_EINVAL
    assert 'at most' in ed.capi.last_error()


def test_noalloc_real_input_bit_identical(setup):
    """A real input (imaginary parts exactly zero) takes ed_ham_apply through
    the real-part gathers; the allocation-free kernel always gathers (re, im)
    pairs.  Both sum the same exact integers and round once, so the results
    must agree bit for bit."""
    import torch
    ed = setup
    lib = ed.capi.lib()
    env = ed.Environment(nspins=20)
    b, h = _ham(ed, env, 20, 4, 5, 0)
    gen = torch.Generator(device='cuda').manual_seed(99)
    x = torch.complex(torch.rand(b.size, dtype=torch.float64, device='cuda', generator=gen) * 2 - 1,
                      torch.zeros(b.size, dtype=torch.float64, device='cuda'))
    y_ref = torch.empty_like(x)
    y_new = torch.empty_like(x)
    assert lib.ed_ham_apply(h.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_ref.data_ptr())) == 0
    rc = lib.ed_ham_apply_noalloc(h.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_new.data_ptr()))
    assert rc == 0, ed.capi.last_error()
    torch.cuda.synchronize()
    assert torch.equal(torch.view_as_real(y_new).view(torch.int64), torch.view_as_real(y_ref).view(torch.int64))
