"""Momentum integrals <a| d/dr |b> (momentum2CIntg, the optical matrix
elements' primitive, src/olcao/gaussIntegrals.f90:23041-39068) on the CPU
oracle, pinned to the reference (no GPU):

* every committed golden block (tests/golden/momentum.npz, evaluated from the
  reference's own generated statements by oracle/fexpr_eval.py) against the
  oracle's restatement, all 16 class pairs s..f and the three components;
* the fixture re-derived from the reference when its source tree is present;
* the semantics: the derivative acts on the ket, <a| d/dx |b> = -d/dB_x <a|b>,
  against a central difference of the overlap primitive.
"""

import os

import numpy as np
import pytest

import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
REF_GAUSS = "/root/reference/src/olcao/gaussIntegrals.f90"


@pytest.fixture(scope="module")
def mom():
    return np.load(os.path.join(HERE, "golden", "momentum.npz"))


def _tolerance(p, lm, ref):
    """1e-11 of the block's largest component, plus the rounding the
    reference's own recursion carries: it forms P - A and P - B from
    P = (a1 A + a2 B) / (a1 + a2), which loses the digits of |A|, |B| against
    the small difference when the exponents are very unequal (its
    prefactor 2 a1 (P - A) then carries ~eps |A| 2 a1 of absolute error per
    overlap unit); at coincident centres the exact value of the odd
    components is zero."""
    a1, a2 = p[0], p[1]
    l1, l2 = lm
    ov = np.abs(orc.primitive(1, p, [l1, l2])[:l1, :l2]).max()
    reach = 1.0 + np.abs(p[3:6]).max() + np.abs(p[6:9]).max()
    return 1e-11 * np.abs(ref[:l1, :l2]).max() + 64 * 2.0 ** -52 * reach * 2.0 * max(a1, a2) * ov


def test_oracle_momentum_matches_reference_goldens(mom):
    for i in range(len(mom["lmalpha"])):
        p = mom["params"][i]
        l1, l2 = (int(x) for x in mom["lmalpha"][i])
        tol = _tolerance(p, (l1, l2), mom["sh"][i])
        for c in range(3):
            got = orc.primitive(6 + c, p, [l1, l2])[:l1, :l2]
            err = np.abs(got - mom["sh"][i][:l1, :l2, c]).max()
            assert err <= tol, f"block {i} lm ({l1},{l2}) component {c}: {err:.2e} > {tol:.2e}"


@pytest.mark.skipif(not os.path.exists(REF_GAUSS), reason="reference tree not present")
def test_momentum_fixture_regenerates_from_reference(mom):
    import fexpr_eval as fe
    F = fe.FortranIntegrals(REF_GAUSS)
    for i in range(0, len(mom["lmalpha"]), 11):
        p = mom["params"][i]
        l1, l2 = (int(x) for x in mom["lmalpha"][i])
        sh = F.momentum(p[0], p[1], p[3:6], p[6:9], fe.l1l2switch(l1, l2))
        np.testing.assert_array_equal(sh[:l1, :l2], mom["sh"][i][:l1, :l2])


@pytest.mark.parametrize("lm", [(1, 1), (4, 9), (9, 4), (16, 16), (1, 16)])
def test_momentum_is_minus_the_derivative_of_the_overlap_in_b(lm):
    rng = np.random.default_rng(7)
    a1, a2 = 0.8, 1.7
    A = rng.normal(size=3)
    B = A + rng.normal(size=3) * 0.7
    h = 1e-5
    for c in range(3):
        Bp, Bm = B.copy(), B.copy()
        Bp[c] += h
        Bm[c] -= h
        fd = -(orc.primitive(1, [a1, a2, 0, *A, *Bp, 0, 0, 0], lm) -
               orc.primitive(1, [a1, a2, 0, *A, *Bm, 0, 0, 0], lm)) / (2 * h)
        got = orc.primitive(6 + c, [a1, a2, 0, *A, *B, 0, 0, 0], lm)
        l1, l2 = lm
        assert np.abs(got[:l1, :l2] - fd[:l1, :l2]).max() <= 1e-7 * max(1.0, np.abs(got).max())
