"""Occupations (olc_populate_states) against the oracle's restatement of
populateStates (src/olcao/populate.F90:132-578), host-only entry, no GPU.

* the reference's merge sort (sortSubs.f90:18-175) as restated: sorted
  output, and ties taken from the second run first;
* standard filling: insulators fill the lowest bands of every k, the last
  electron fraction and the even spread over a degenerate top level;
* thermal smearing: the bisection's Fermi energy and Fermi-Dirac weights;
* spin 2, the structured (state, k, spin) layout, and the error when the
  states cannot hold the electrons.
"""

import numpy as np
import pytest

import oracle as orc


def _c(gpu_free_lib, ev, kw, ne, **kw2):
    from olcao_gb300 import api
    return api.populate_states(ev, kw, ne, **kw2)


def test_merge_sort_restatement():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 7, 16, 33, 100):
        v = list(np.round(rng.normal(size=n), 1))          # many ties
        s, o = orc.merge_sort(v)
        assert s == sorted(v)
        assert [v[i] for i in o] == s
    # ties: the element of the second run comes first
    s, o = orc.merge_sort([1.0, 1.0])
    assert o == [1, 0]


@pytest.mark.parametrize("spin", [1, 2])
@pytest.mark.parametrize("sigma", [0.0, 0.003])
def test_populate_matches_oracle(gpu_free_lib, spin, sigma):
    rng = np.random.default_rng(10 * spin + int(sigma * 1000))
    nk, ns = 5, 12
    ev = np.sort(rng.normal(size=(spin, nk, ns)), axis=2)
    kw = np.full(nk, 2.0 / nk)
    ne = 9.3                                               # metallic filling
    occ, ef = _c(gpu_free_lib, ev, kw, ne, thermal_sigma=sigma)
    ro, ref_ef = orc.populate_states(ev, kw, ne, thermal_sigma=sigma)
    np.testing.assert_allclose(occ, ro, rtol=1e-14, atol=1e-15)
    assert ef == pytest.approx(ref_ef, rel=1e-14, abs=1e-15)
    assert occ.sum() == pytest.approx(ne, abs=1e-8)
    assert (occ >= 0).all() and (occ <= kw[None, :, None] / spin + 1e-15).all()


def test_insulator_fills_lowest_bands(gpu_free_lib):
    rng = np.random.default_rng(5)
    nk, ns, nocc = 8, 10, 4
    base = np.sort(rng.uniform(-2.0, -1.0, (nk, nocc)), axis=1)
    cond = np.sort(rng.uniform(0.5, 1.5, (nk, ns - nocc)), axis=1)
    ev = np.concatenate([base, cond], axis=1)
    kw = np.full(nk, 2.0 / nk)
    occ, ef = _c(gpu_free_lib, ev, kw, 2.0 * nocc)
    np.testing.assert_allclose(occ[:, :nocc], 2.0 / nk, rtol=1e-14)
    assert (occ[:, nocc:] == 0).all()
    assert ef == base.max()
    # smeared: Fermi level inside the gap, same occupations
    occ2, ef2 = _c(gpu_free_lib, ev, kw, 2.0 * nocc, thermal_sigma=0.001)
    assert base.max() < ef2 < cond.min()
    np.testing.assert_allclose(occ2, occ, atol=1e-12)


def test_degenerate_top_level_shares_charge(gpu_free_lib):
    # three states at -0.2 across k-points hold 1 of their possible 3 electrons
    ev = np.array([[-1.0, -0.2, 0.5], [-1.0, -0.2, 0.5], [-1.0, -0.2 + 5e-9, 0.5]])
    kw = np.full(3, 2.0 / 3)
    occ, ef = _c(gpu_free_lib, ev, kw, 3.0)
    ro, _ = orc.populate_states(ev[None], kw, 3.0)
    np.testing.assert_allclose(occ, ro[0], rtol=1e-14)
    np.testing.assert_allclose(occ[:, 1], 1.0 / 3, rtol=1e-12)
    assert occ.sum() == pytest.approx(3.0, abs=1e-12)


def test_too_many_electrons_is_an_error(gpu_free_lib):
    from olcao_gb300 import api
    with pytest.raises(api.OlcError):
        api.populate_states(np.zeros((2, 3)), np.full(2, 1.0), 7.0)

