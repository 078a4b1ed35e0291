"""Parity of the CUDA integral path with the CPU oracle (gpu).

Each operator pass (gaussOverlapOL/KE/NP/EP of src/olcao/integrals.F90) is
compared block by block -- valeVale, coreVale, coreCore for every k -- and
after orthogonalisation and packing, on small seeded systems the oracle runs
in seconds.  Tolerance: 1e-10 relative to the largest magnitude of the k-block
(the FP64 path's integral bar).
"""

import numpy as np
import pytest

import oracle as orc
from olcao_gb300 import system as S

RTOL = 1e-10

SYSTEMS = {
    "c2": lambda: S.small_test_system("c2", nk=(2, 2, 2)),
    "si2": lambda: S.small_test_system("si2", nk=(2, 2, 2)),
    "sio": lambda: S.small_test_system("sio", nk=(2, 1, 2)),
    "sif": lambda: S.small_test_system("sif", nk=(2, 1, 2)),
}


def _cmp(gpu, ref, what):
    g = gpu.cpu().numpy() if hasattr(gpu, "cpu") else gpu
    for k in range(ref.shape[0]):
        scale = max(np.abs(ref[k]).max(), 1e-300)
        err = np.abs(g[k] - ref[k]).max()
        assert err <= RTOL * scale + 1e-14, f"{what} k={k}: err {err:.3e} scale {scale:.3e}"


@pytest.fixture(scope="module", params=sorted(SYSTEMS))
def pair(request, gpu_lib):
    from olcao_gb300 import api
    sysm = SYSTEMS[request.param]()
    return sysm, orc.Oracle(sysm), api.Context(sysm)


@pytest.mark.gpu
@pytest.mark.parametrize("op", [1, 2, 3])
def test_operator_blocks(pair, op):
    sysm, o, ctx = pair
    vv, cv, cc = ctx.gauss_overlap(op)
    rv, rc, rcc = o.operator(op)
    _cmp(vv, rv, f"op{op} valeVale")
    if o.core_dim:
        _cmp(cv, rc, f"op{op} coreVale")
        _cmp(cc, rcc, f"op{op} coreCore")


@pytest.mark.gpu
def test_elecpot_terms(pair):
    sysm, o, ctx = pair
    for term in sorted({0, o.pot_dim // 2, o.pot_dim - 1}):
        vv, cv, cc = ctx.gauss_overlap(4, term)
        rv, rc, rcc = o.operator(4, term)
        _cmp(vv, rv, f"EP{term} valeVale")
        if o.core_dim:
            _cmp(cv, rc, f"EP{term} coreVale")
            _cmp(cc, rcc, f"EP{term} coreCore")


@pytest.mark.gpu
def test_ortho_pack(pair):
    sysm, o, ctx = pair
    vS, cS, ccS = ctx.gauss_overlap(1)
    rS, rcS, rccS = o.operator(1)
    pS = ctx.ortho_pack(True, vS.clone(), cS, ccS, cS)
    _cmp(pS, o.ortho_pack(True, rS, rcS, rccS, rcS), "packed S")
    vK, cK, ccK = ctx.gauss_overlap(2)
    rK, rcK, rccK = o.operator(2)
    pK = ctx.ortho_pack(False, vK, cK, ccK, cS)
    _cmp(pK, o.ortho_pack(False, rK, rcK, rccK, rcS), "packed KE")


@pytest.mark.gpu
def test_hamiltonian_fused_equals_sum(pair):
    """OLC_OP_HAMILTONIAN (KE + NP + sum c_j V_j in one pass) equals the sum
    of the separate passes (linearity of the integral pass)."""
    sysm, o, ctx = pair
    c = sysm.pot_coeffs
    hv, hc, hcc = ctx.gauss_overlap(6, coeffs=c)
    acc = [x.cpu().numpy().copy() if x is not None else None for x in ctx.gauss_overlap(2)]
    for op in (3,):
        r = ctx.gauss_overlap(op)
        for i in range(3):
            if acc[i] is not None:
                acc[i] += r[i].cpu().numpy()
    for j in range(o.pot_dim):
        r = ctx.gauss_overlap(4, j)
        for i in range(3):
            if acc[i] is not None:
                acc[i] += c[j] * r[i].cpu().numpy()
    _cmp(hv, acc[0], "fused H valeVale")
    if o.core_dim:
        _cmp(hc, acc[1], "fused H coreVale")
        _cmp(hcc, acc[2], "fused H coreCore")


@pytest.mark.gpu
def test_elecpot_far_shell_fp32_matches_fp64(pair):
    """Mixed precision evaluates images past the far-shell cut in FP32; the
    blocks stay within the FP64 bar of the oracle."""
    from olcao_gb300 import api
    sysm, o, ctx = pair
    for term in sorted({0, o.pot_dim - 1}):
        vv, cv, cc = ctx.gauss_overlap(4, term, precision=api.PREC_MIXED)
        rv, rc, rcc = o.operator(4, term)
        _cmp(vv, rv, f"EP{term} mixed valeVale")
        if o.core_dim:
            _cmp(cv, rc, f"EP{term} mixed coreVale")
            _cmp(cc, rcc, f"EP{term} mixed coreCore")
