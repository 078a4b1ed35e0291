"""Valence density and traces on the GPU (olc_make_valence_rho) vs the
oracle's makeValenceRho restatement (gpu).

The GPU's own eigenvectors are handed to both sides, so the comparison
covers the density and trace step alone; the operators are the oracle's
packed S, NP, KE, V_j on one side and the GPU's prepared ones on the other,
which agree to 1e-10 of their largest element, so a trace may differ by
2e-10 max|T| sum|rho| (written into each check).  At the Si64 size the
traces are checked against sum f x^H S x and sum f x^H H x formed from the
prepared S(k), H(k), and, for FP64 eigenpairs, against the identities the
reference prints after the traces (valeCharge.F90:432-470): <psi|psi> =
number of electrons, and Electron Sum = Electron Energy.
"""

import numpy as np
import pytest

import oracle as orc
from olcao_gb300 import system as S

SYSTEMS = {
    "c2": lambda: S.small_test_system("c2", nk=(2, 2, 2)),
    "sio": lambda: S.small_test_system("sio", nk=(2, 1, 2)),
}


@pytest.fixture(scope="module", params=sorted(SYSTEMS))
def case(request, gpu_lib):
    from olcao_gb300 import api
    sysm = SYSTEMS[request.param]()
    o = orc.Oracle(sysm)
    packed = o.packed_operators()
    ctx = api.Context(sysm)
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
    return sysm, o, packed, ctx


def _channels(ctx, sysm, spin, seed):
    """Eigenpairs of `spin` channels (coefficients scaled per channel) and
    occupations with empty states and entries under smallThresh."""
    import torch
    from olcao_gb300 import api
    n, nk = ctx.vale_dim, ctx.nk
    rng = np.random.default_rng(seed)
    vecs = torch.zeros(spin, nk, n, n, dtype=torch.complex128, device="cuda")
    eig = np.zeros((spin, nk, n))
    for s in range(spin):
        eig[s] = ctx.scf_iteration(sysm.pot_coeffs * (1.0 + 0.1 * s), n, precision=api.PREC_FP64,
                                   vectors=vecs[s])
    occ = rng.uniform(0.0, 2.0 / nk, (spin, nk, n))
    occ[:, :, n // 2:] = 0.0
    occ[:, 0, 1] = 3e-9                  # left out: below smallThresh in every channel
    if spin == 2:
        occ[1, :, 0] = 0.0               # empty in one channel only: kept
    return occ, eig, vecs


@pytest.mark.gpu
@pytest.mark.parametrize("spin", [1, 2])
def test_valence_rho_matches_oracle(case, spin):
    sysm, o, packed, ctx = case
    occ, eig, vecs = _channels(ctx, sysm, spin, seed=spin)
    traces, energy, rho = ctx.make_valence_rho(occ, vecs, eig, rho=True)
    rt, re_, rrho = orc.make_valence_rho(packed, o.pot_dim, occ, eig, vecs.cpu().numpy())
    got = rho.cpu().numpy()
    assert np.abs(got - rrho).max() <= 1e-12 * np.abs(rrho).max()
    names = ["S", "NP", "KE"] + [f"V{j}" for j in range(o.pot_dim)]
    rsum = np.abs(rrho).sum(axis=(1, 2, 3))                      # per spin column
    for t, name in enumerate(names):
        bound = 2e-10 * np.abs(packed[name]).max() * rsum + 1e-12 * np.abs(rt[:, t])
        assert (np.abs(traces[:, t] - rt[:, t]) <= bound).all(), (name, traces[:, t], rt[:, t])
    assert np.allclose(energy, re_, rtol=1e-13, atol=0)


@pytest.mark.gpu
def test_fused_form_traces_match_stored(case, gpu_lib):
    from olcao_gb300 import api
    sysm, o, packed, ctx = case
    occ, eig, vecs = _channels(ctx, sysm, 2, seed=7)
    ts, es, _ = ctx.make_valence_rho(occ, vecs, eig)
    cf = api.Context(sysm)
    cf.scf_prepare(api.PREC_FP64, api.FORM_FUSED)
    tf, ef, _ = cf.make_valence_rho(occ, vecs, eig)
    assert np.allclose(tf, ts, rtol=1e-11, atol=1e-12 * np.abs(ts).max())
    assert np.array_equal(ef, es)
    cf.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_si64_traces(gpu_lib, precision):
    """Si64 (832 basis functions, every 8th of the 64 k), insulator
    occupation 2/nk on the 128 lowest states.  Whatever the vectors' quality,
    tr(rho S) = sum f x^H S x and, by linearity, sum_t c_t tr(rho T_t) =
    sum f x^H H x with the prepared S(k) and H(k); checked to FP64 rounding.
    With FP64 eigenpairs these are also the reference's printed identities:
    the electron count, and Electron Sum = Electron Energy."""
    import torch
    from olcao_gb300 import api
    sysm = S.SYSTEMS["si64"]()
    sysm.kpoints_abc = sysm.kpoints_abc[::8]
    ctx = api.Context(sysm)
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
    n, nk = ctx.vale_dim, ctx.nk
    prec = api.PREC_MIXED if precision == "mixed" else api.PREC_FP64
    vec = torch.zeros(nk, n, n, dtype=torch.complex128, device="cuda")
    w = ctx.scf_iteration(sysm.pot_coeffs, n, precision=prec, vectors=vec)
    nocc = 2 * len(sysm.site_type)
    occ = np.zeros((nk, n))
    occ[:, :nocc] = 2.0 / nk
    traces, energy, _ = ctx.make_valence_rho(occ, vec, w)
    X = vec.cpu().numpy()
    exp_s = exp_h = 0.0
    for k in range(nk):
        H, Sm = ctx.scf_matrices(sysm.pot_coeffs, k)
        Z = X[k, :nocc].T                                   # [n, nocc]
        f = occ[k, :nocc]
        exp_s += (f * np.einsum("ij,ij->j", Z.conj(), Sm @ Z).real).sum()
        exp_h += (f * np.einsum("ij,ij->j", Z.conj(), H @ Z).real).sum()
    c = np.where(sysm.pot_coeffs == 0.0, 1.0, sysm.pot_coeffs)
    parts = np.concatenate([[traces[0, 1], traces[0, 2]], c * traces[0, 3:]])
    esum = parts.sum()
    assert abs(traces[0, 0] - exp_s) <= 1e-11 * exp_s
    assert abs(esum - exp_h) <= 1e-11 * np.abs(parts).sum(), (esum, exp_h)
    if precision == "fp64":
        electrons = occ.sum()
        assert abs(traces[0, 0] - electrons) <= 1e-9 * electrons
        assert abs(esum - energy[0]) <= 1e-8 * electrons, (esum, energy[0])
