"""Scalar-relativistic path (rel = 1) on the GPU vs the oracle (gpu).

The mass-velocity operator (gaussOverlapMV, integrals.F90:904-1320) is
orthogonalised and packed like the kinetic energy and joins H(k) with factor
1 (secularEqn.F90:137-143).  Checked: the packed MV operator against the
oracle's (1e-10 of the largest element, the bar of the other operators), the
eigenvalues of the stored and fused SCF passes against LAPACK zhegv on the
oracle's H(k) (1e-8 Ha), the massVelocityTrace of the density step, and the
atomMVOverlap datasets of the setup writer.
"""

import numpy as np
import pytest

import oracle as orc
from olcao_gb300 import system as S

EIG_TOL = 1e-8


@pytest.fixture(scope="module", params=["si2", "sio", "sif"])
def case(request, gpu_lib):
    from olcao_gb300 import api
    sysm = S.small_test_system(request.param, nk=(2, 1, 2))
    sysm.rel = 1
    o = orc.Oracle(sysm)
    packed = o.packed_operators()
    assert "MV" in packed
    hp = orc.assemble(packed, sysm.pot_coeffs)
    w, vec = orc.zhegv(hp, packed["S"], o.vale_dim, o.vale_dim)
    return sysm, o, packed, w, api.Context(sysm)


@pytest.mark.gpu
def test_massvel_operator_matches_oracle(case):
    sysm, o, packed, w, ctx = case
    gp = ctx.packed_operators(terms=[0])
    ref = packed["MV"]
    got = gp["MV"].cpu().numpy()
    assert np.abs(ref).max() > 0
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max() + 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["stored", "fused"])
def test_relativistic_scf_pass_matches_oracle(case, form):
    from olcao_gb300 import api
    sysm, o, packed, w, ctx = case
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED if form == "stored" else api.FORM_FUSED)
    eig = ctx.scf_iteration(sysm.pot_coeffs, o.vale_dim, precision=api.PREC_FP64)
    err = np.abs(eig - w).max()
    assert err <= EIG_TOL, f"{form}: max eigenvalue error {err:.2e} Ha"
    # the mass velocity is not negligible in these tests
    c0 = sysm.pot_coeffs.copy()
    nonrel = orc.zhegv(orc.assemble({k: v for k, v in packed.items() if k != "MV"}, c0),
                       packed["S"], o.vale_dim, o.vale_dim)[0]
    assert np.abs(nonrel - w).max() > 100 * EIG_TOL


@pytest.mark.gpu
def test_massvel_trace_and_writer(case, tmp_path):
    import torch
    from olcao_gb300 import api
    sysm, o, packed, w, ctx = case
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
    n, nk = ctx.vale_dim, ctx.nk
    vec = torch.zeros(nk, n, n, dtype=torch.complex128, device="cuda")
    eig = ctx.scf_iteration(sysm.pot_coeffs, n, precision=api.PREC_FP64, vectors=vec)
    occ = np.zeros((nk, n))
    occ[:, : n // 3] = 2.0 / nk
    tr, en, _ = ctx.make_valence_rho(occ, vec, eig)
    assert tr.shape == (1, 4 + o.pot_dim)
    rt, re_, rrho = orc.make_valence_rho(packed, o.pot_dim, occ[None], eig[None], vec.cpu().numpy()[None])
    names = ["S", "NP", "KE", "MV"] + [f"V{j}" for j in range(o.pot_dim)]
    rsum = np.abs(rrho).sum()
    for t, name in enumerate(names):
        bound = 2e-10 * np.abs(packed[name]).max() * rsum + 1e-12 * abs(rt[0, t])
        assert abs(tr[0, t] - rt[0, t]) <= bound, (name, tr[0, t], rt[0, t])
    # Electron Sum with the mass velocity (valeCharge.F90:448-452)
    c = np.where(sysm.pot_coeffs == 0.0, 1.0, sysm.pot_coeffs)
    esum = (c * tr[0, 4:]).sum() + tr[0, 1] + tr[0, 2] + tr[0, 3]
    assert abs(esum - en[0]) <= 1e-8 * occ.sum()
    root = str(tmp_path / "setup")
    ctx.write_setup_integrals(root)
    mv = api.read_dataset(root, "/atomIntgGroup/atomMVOverlap/0000001")
    np.testing.assert_allclose(mv.T, packed["MV"][0], rtol=0, atol=1e-10 * np.abs(packed["MV"]).max() + 1e-14)
