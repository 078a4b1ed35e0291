"""Valence density and traces: the oracle's restatement of makeValenceRho
(src/olcao/valeCharge.F90:172-395) checked on the CPU.

* matrix_element_mult against a loop that follows matrixSubs.F90:39-51
  element by element;
* the identities the reference prints after the traces (valeCharge.F90:
  432-470): <psi|psi> = sum of the kept occupations, and the "Electron Sum"
  sum_j c_j potRho_j + KE + NP equals the "Electron Energy" sum f * lambda
  for exact eigenpairs of H = NP + KE + sum_j c_j V_j;
* spin 2: the columns are the traces of up + down and up - down;
* states with sum_s |f| below smallThresh are left out.
"""

import numpy as np
import pytest
import scipy.linalg as sl

import oracle as orc


def _reference_loop(m1, m2, n):
    """matrixSubs.F90:39-51, index by index (0-based)."""
    temp = 0.0
    diagonal = -1
    for i in range(1, n + 1):
        for j in range(diagonal + 1, diagonal + i):
            temp += m1[j, 0] * m2[j, 0] + m1[j, 1] * m2[j, 1]
        diagonal += i
        temp += m1[diagonal, 0] * m2[diagonal, 0] / 2.0
    return 2.0 * temp


def _random_hermitian_packed(rng, n, shift=0.0):
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    h = (a + a.conj().T) / 2 + shift * np.eye(n)
    rows, cols = orc.packed_index(n)
    v = h[rows, cols]
    return np.stack([v.real, v.imag], -1)


@pytest.mark.parametrize("n", [1, 2, 7, 12])
def test_matrix_element_mult_follows_reference_loop(n):
    rng = np.random.default_rng(n)
    plen = n * (n + 1) // 2
    a = rng.standard_normal((plen, 2))
    b = rng.standard_normal((plen, 2))
    assert orc.matrix_element_mult(a, b) == pytest.approx(_reference_loop(a, b, n), rel=1e-13, abs=1e-13)


def _problem(seed, n=9, nk=3, pot_dim=3, spin=1):
    rng = np.random.default_rng(seed)
    packed = {"S": np.stack([_random_hermitian_packed(rng, n, shift=3 * n) / n for _ in range(nk)])}
    for name in ["NP", "KE"] + [f"V{j}" for j in range(pot_dim)]:
        packed[name] = np.stack([_random_hermitian_packed(rng, n) for _ in range(nk)])
    chans = []
    for s in range(spin):
        c = rng.standard_normal(pot_dim) * 0.3
        c[0] = 0.0                          # the zero-coefficient rule
        hp = orc.assemble(packed, c)
        w, vec = orc.zhegv(hp, packed["S"], n, n)
        chans.append((c, w, vec))
    occ = rng.uniform(0.0, 2.0, (spin, nk, n))
    occ[:, :, -2:] = 0.0                    # empty states
    occ[:, 1, 3] = 2e-9                     # below smallThresh in every channel
    eig = np.stack([ch[1] for ch in chans])
    vectors = np.stack([ch[2].transpose(0, 2, 1) for ch in chans])     # [spin, nk, state, n]
    return packed, chans, occ, eig, vectors


def test_traces_satisfy_reference_identities():
    pot_dim = 3
    packed, chans, occ, eig, vectors = _problem(5, pot_dim=pot_dim)
    traces, energy, rho = orc.make_valence_rho(packed, pot_dim, occ, eig, vectors)
    kept = occ.copy()
    kept[np.abs(occ).sum(0)[None].repeat(occ.shape[0], 0) < orc.SMALL_THRESH] = 0.0
    # <psi|psi> = number of electrons
    assert traces[0, 0] == pytest.approx(kept.sum(), rel=1e-12)
    # Electron Sum = Electron Energy
    c = np.where(chans[0][0] == 0.0, 1.0, chans[0][0])
    esum = (c * traces[0, 3:]).sum() + traces[0, 1] + traces[0, 2]
    assert esum == pytest.approx(energy[0], rel=1e-11)
    assert energy[0] == pytest.approx((kept * eig).sum(), rel=1e-13)
    # packed rho is the upper triangle of sum_n f x x^H
    k = 2
    X = vectors[0, k].T
    R = (X * kept[0, k][None, :]) @ X.conj().T
    rows, cols = orc.packed_index(X.shape[0])
    assert np.abs(rho[0, k, :, 0] + 1j * rho[0, k, :, 1] - R[rows, cols]).max() < 1e-13


def test_spin_two_columns_are_total_and_difference():
    pot_dim = 2
    packed, chans, occ, eig, vectors = _problem(6, pot_dim=pot_dim, spin=2)
    traces, energy, rho = orc.make_valence_rho(packed, pot_dim, occ, eig, vectors)
    up = orc.make_valence_rho(packed, pot_dim, occ[:1], eig[:1], vectors[:1])
    dn = orc.make_valence_rho(packed, pot_dim, occ[1:], eig[1:], vectors[1:])
    # the kept set is common to both channels; state 3 of k 1 is below the
    # threshold in both, so the per-channel runs keep the same states
    assert np.allclose(traces[0], up[0][0] + dn[0][0], rtol=1e-12, atol=1e-12)
    assert np.allclose(traces[1], up[0][0] - dn[0][0], rtol=1e-12, atol=1e-12)
    assert np.allclose(energy, [up[1][0], dn[1][0]], rtol=1e-13)
    assert np.allclose(rho[0], up[2][0] + dn[2][0], atol=1e-13)
    # the reference's spin-resolved Electron Sum (valeCharge.F90:472-508)
    for s, sign in ((0, 1.0), (1, -1.0)):
        c = np.where(chans[s][0] == 0.0, 1.0, chans[s][0])
        esum = 0.5 * ((c * (traces[0, 3:] + sign * traces[1, 3:])).sum()
                      + traces[0, 2] + sign * traces[1, 2] + traces[0, 1] + sign * traces[1, 1])
        assert esum == pytest.approx(energy[s], rel=1e-11)


def test_make_valence_rho_rejects_bad_arguments(gpu_free_lib):
    from olcao_gb300 import api
    tr = np.zeros(8)
    occ = np.ones(4)
    st = gpu_free_lib.olc_make_valence_rho(None, 2, 1, occ.ctypes.data, None, None, tr.ctypes.data,
                                           None, None)
    assert st == 1
    assert "null context" in api.last_error()
