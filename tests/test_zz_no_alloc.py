"""The allocation-free eigen-solve entry point (gpu).

olc_solve_zhegv_noalloc serves callers that may not allocate device memory
once their SCF loop runs (a host that gives all device memory to its own pool
at start-up, or a framework that owns the allocator).  It solves from packed
H(k), S(k) using a fixed 16 MiB device array as working space.  Here it is
called through the C ABI twice in a row and must agree with the ordinary
olc_solve_zhegv on the same matrices, to the 1e-8 Ha eigenvalue bar the
other solver tests use; sizes beyond its working array are refused.

This file is collected last so that a failure here never hides another test.
"""

import ctypes as C

import numpy as np
import pytest

from olcao_gb300 import system as S

EIG_TOL = 1e-8


def _packed_case():
    import torch
    from olcao_gb300 import api
    sysm = S.small_test_system("tiny", nk=(1, 2, 2))
    ctx = api.Context(sysm)
    packed = ctx.packed_operators()
    H = ctx.assemble_hamiltonian(packed, sysm.pot_coeffs)
    return ctx, H.contiguous(), packed["S"].contiguous(), torch


def _noalloc(lib, n, nk, H, Sm, torch, nstates):
    eig = torch.zeros(nk, nstates, dtype=torch.float64, device="cuda")
    vec = torch.zeros(nk, nstates, n, dtype=torch.complex128, device="cuda")
    info = torch.full((nk,), -1, dtype=torch.int32, device="cuda")
    st = lib.olc_solve_zhegv_noalloc(n, nk, H.data_ptr(), Sm.data_ptr(), nstates,
                                     eig.data_ptr(), vec.data_ptr(), info.data_ptr(),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, eig.cpu().numpy(), vec.cpu().numpy(), info.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_solver_matches_the_allocating_solver_twice(gpu_lib):
    from olcao_gb300 import api
    ctx, H, Sm, torch = _packed_case()
    n, nk = ctx.vale_dim, ctx.nk
    lib = api.lib()
    for scale in (1.0, 0.5):           # two calls in a row, different data
        Hs = (H * scale).contiguous()
        ref, _, info_ref = ctx.solve_zhegv(Hs, Sm, n)
        st, eig, vec, info = _noalloc(lib, n, nk, Hs, Sm, torch, n)
        assert st == 0, api.last_error()
        assert (info == 0).all() and (info_ref == 0).all()
        assert np.abs(eig - ref.cpu().numpy()).max() <= EIG_TOL
        # vectors are S-orthonormal and solve the pencil; eigenvalues also
        # against LAPACK, which shares no code with either device solver
        import oracle as orc
        import scipy.linalg as sl
        Sp, Hp = Sm.cpu().numpy(), Hs.cpu().numpy()
        for k in range(nk):
            Sk, Hk = orc.unpack(Sp[k], n), orc.unpack(Hp[k], n)
            Z = vec[k].T
            assert np.abs(Z.conj().T @ Sk @ Z - np.eye(n)).max() < 1e-9
            assert np.abs(Hk @ Z - Sk @ Z * eig[k][None, :]).max() < 1e-8 * max(1.0, np.abs(Hk).max())
            assert np.abs(eig[k] - sl.eigh(Hk, Sk, eigvals_only=True)).max() <= EIG_TOL


@pytest.mark.gpu
def test_noalloc_solver_allocates_no_device_memory(gpu_lib):
    """After a first call (which looks up the working array's address), more
    calls leave the free device memory unchanged."""
    from olcao_gb300 import api
    ctx, H, Sm, torch = _packed_case()
    n, nk = ctx.vale_dim, ctx.nk
    lib = api.lib()
    eig = torch.zeros(nk, n, dtype=torch.float64, device="cuda")
    vec = torch.zeros(nk, n, n, dtype=torch.complex128, device="cuda")
    info = torch.zeros(nk, dtype=torch.int32, device="cuda")
    args = (n, nk, H.data_ptr(), Sm.data_ptr(), n, eig.data_ptr(), vec.data_ptr(), info.data_ptr(), None)
    assert lib.olc_solve_zhegv_noalloc(*args) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert lib.olc_solve_zhegv_noalloc(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


@pytest.mark.gpu
def test_noalloc_solver_refuses_sizes_beyond_its_array(gpu_lib):
    import torch
    from olcao_gb300 import api
    lib = api.lib()
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    info = torch.zeros(16, dtype=torch.int32, device="cuda")
    st = lib.olc_solve_zhegv_noalloc(65, 1, d.data_ptr(), d.data_ptr(), 1, d.data_ptr(),
                                     None, info.data_ptr(), None)
    msg = api.last_error()
    assert st == 1 and "n exceeds 64" in msg
    st = lib.olc_solve_zhegv_noalloc(64, 129, d.data_ptr(), d.data_ptr(), 1, d.data_ptr(),
                                     None, info.data_ptr(), None)
    msg = api.last_error()
    assert st == 1 and "exceeds" in msg and "working array" in msg
