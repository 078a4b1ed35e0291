"""Mixed-precision path (gpu).

* olc_split_zgemm: the error-free split-BF16 complex product must agree with
  an FP64 product to FP64 rounding;
* OLC_PREC_MIXED eigen-solve (FP32 solve + Rayleigh-Ritz with split products)
  against the plain FP64 GPU path on the same H(k), S(k): eigenvalues within
  1e-6 Ha (the mixed-form bar), band energy within 1e-5 Ha, vectors
  S-orthonormal with small residuals.
"""

import numpy as np
import pytest

from olcao_gb300 import system as S

MIXED_EIG_TOL = 1e-6
BAND_TOL = 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,k", [(40, 33, 17), (64, 64, 300), (31, 90, 1500), (200, 260, 2100)])
def test_split_zgemm_is_fp64_accurate(gpu_lib, m, n, k):
    import torch
    from olcao_gb300 import api
    rng = np.random.default_rng(m + n + k)
    A = (rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k)))
    A *= np.exp(rng.uniform(-20, 20, (m, 1)))           # rows of very different scale
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n)))
    B *= np.exp(rng.uniform(-5, 5, (1, n)))
    ctx = api.Context(S.small_test_system("tiny", nk=(1, 1, 1)))
    C = ctx.split_zgemm(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()).cpu().numpy()
    ref = A @ B
    # error bounded by FP64 rounding of |A||B| (per row/column scale)
    bound = 4 * k * 2.0 ** -52 * (np.abs(A) @ np.abs(B))
    assert (np.abs(C - ref) <= bound + 1e-300).all()


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,k,conj", [(40, 33, 17, False), (130, 300, 257, True),
                                        (257, 129, 1000, False), (832, 832, 832, True)])
def test_split_cgemm32_is_fp32_accurate(gpu_lib, m, n, k, conj):
    """Tensor-core product from three BF16 pieces per FP32 operand: within
    FP32 rounding of |op(A)| |B| (element by element)."""
    import torch
    from olcao_gb300 import api
    rng = np.random.default_rng(m * 7 + n + k)
    shape_a = (k, m) if conj else (m, k)
    A = (rng.standard_normal(shape_a) + 1j * rng.standard_normal(shape_a)).astype(np.complex64)
    A *= np.exp(rng.uniform(-3, 3, (shape_a[0], 1))).astype(np.float32)
    B = (rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))).astype(np.complex64)
    ctx = api.Context(S.small_test_system("tiny", nk=(1, 1, 1)))
    C = ctx.split_cgemm32(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), conj_a=conj).cpu().numpy()
    Ad = A.astype(np.complex128)
    opA = Ad.conj().T if conj else Ad
    ref = opA @ B.astype(np.complex128)
    # three pieces keep 24 bits; FP32 accumulation adds ~sqrt(K) roundings
    bound = (8 + 2 * np.sqrt(2 * k)) * 2.0 ** -24 * (np.abs(opA) @ np.abs(B.astype(np.complex128))) + 1e-30
    assert (np.abs(C - ref) <= bound).all(), float((np.abs(C - ref) / bound).max())


def _band_energy(w, nocc):
    return 2.0 * w[:, :nocc].sum() / w.shape[0]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["si8", "si64"])
def test_mixed_solver_matches_fp64_path(gpu_lib, name):
    import torch
    from olcao_gb300 import api
    sysm = S.SYSTEMS[name]()
    if name == "si8":
        sysm.kpoints_abc = sysm.kpoints_abc[:8]
    else:
        sysm.kpoints_abc = sysm.kpoints_abc[::8]
    ctx = api.Context(sysm)
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
    n, nk = ctx.vale_dim, ctx.nk
    assert n > 64
    w64 = ctx.scf_iteration(sysm.pot_coeffs, n, precision=api.PREC_FP64)
    vec = torch.zeros(nk, n, n, dtype=torch.complex128, device="cuda")
    wm = ctx.scf_iteration(sysm.pot_coeffs, n, precision=api.PREC_MIXED, vectors=vec)
    err = np.abs(wm - w64).max()
    assert err <= MIXED_EIG_TOL, f"max eigenvalue error {err:.3e} Ha"
    nocc = 2 * len(sysm.site_type)       # 4 valence electrons per Si atom, 2 per state
    assert abs(_band_energy(wm, nocc) - _band_energy(w64, nocc)) <= BAND_TOL
    X = vec.cpu().numpy()
    for k in (0, nk - 1):
        H, Sm = ctx.scf_matrices(sysm.pot_coeffs, k)
        Z = X[k].T
        G = Z.conj().T @ Sm @ Z
        assert np.abs(G - np.eye(n)).max() < 1e-4
        R = H @ Z - Sm @ Z * wm[k][None, :]
        assert np.abs(R).max() < 1e-3


@pytest.mark.gpu
def test_graph_replay_matches_direct_pass(gpu_lib):
    """OLC_ITER_GRAPH: direct first call, capture on the second, replays
    after; every call gives the direct pass's eigenvalues for its inputs
    (within the mixed path's run-to-run spread: the FP32 reduction sums with
    shared-memory atomics) and launches the same number of kernels of this
    library."""
    import torch
    from olcao_gb300 import api
    sysm = S.SYSTEMS["si8"]()
    sysm.kpoints_abc = sysm.kpoints_abc[:16]
    ctx = api.Context(sysm)
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
    n = ctx.vale_dim
    vec = torch.zeros(ctx.nk, n, n, dtype=torch.complex128, device="cuda")
    coeffs = [sysm.pot_coeffs * f for f in (1.0, 0.97, 1.02, 1.0)]
    direct = [ctx.scf_iteration(c, n, precision=api.PREC_MIXED, vectors=vec) for c in coeffs]
    l0 = api.launch_count()
    ctx.scf_iteration(coeffs[0], n, precision=api.PREC_MIXED, vectors=vec)
    per_pass = api.launch_count() - l0
    for i, c in enumerate(coeffs):
        l0 = api.launch_count()
        w = ctx.scf_iteration(c, n, precision=api.PREC_MIXED, vectors=vec, graph=True)
        assert np.abs(w - direct[i]).max() <= 1e-7
        if i >= 1:                     # captured and replayed
            assert api.launch_count() - l0 == per_pass
