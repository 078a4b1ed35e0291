"""Analytic primitives against direct quadrature (the reference's own check:
src/scripts/osrecurintgnum.py, gaussIntgTest.f90).

Each Cartesian Gaussian factorises per direction, so every two- and
three-centre integral of products of Gaussians and polynomials is a sum of
products of 1-D integrals.  Here those 1-D integrals are taken by
Gauss-Hermite quadrature around the product centre, and the derivative
operators (-1/2 d2 for the kinetic energy, (alpha^2/8) nabla^4 for the mass
velocity) are applied to the 1-D functions symbolically (sympy), so no
recurrence and no formula of the primitives is reused.  The real harmonics
are the unnormalised sh components of gaussIntegrals.f90:46-48.  Checked:
the oracle's primitives (which match the reference's generated code) and the
reference goldens, to 1e-10 of each block's largest element.
"""

import math

import numpy as np
import pytest

import oracle as orc

sp = pytest.importorskip("sympy")

# sh components as (coefficient, (ex, ey, ez)) monomials, lm = 1..16
HARM = [
    [(1, (0, 0, 0))], [(1, (1, 0, 0))], [(1, (0, 1, 0))], [(1, (0, 0, 1))],
    [(1, (1, 1, 0))], [(1, (1, 0, 1))], [(1, (0, 1, 1))],
    [(1, (2, 0, 0)), (-1, (0, 2, 0))], [(2, (0, 0, 2)), (-1, (2, 0, 0)), (-1, (0, 2, 0))],
    [(1, (1, 1, 1))], [(1, (2, 0, 1)), (-1, (0, 2, 1))], [(1, (3, 0, 0)), (-3, (1, 2, 0))],
    [(3, (2, 1, 0)), (-1, (0, 3, 0))], [(2, (0, 0, 3)), (-3, (2, 0, 1)), (-3, (0, 2, 1))],
    [(4, (1, 0, 2)), (-1, (3, 0, 0)), (-1, (1, 2, 0))], [(4, (0, 1, 2)), (-1, (2, 1, 0)), (-1, (0, 3, 0))],
]
FINE = 7.2973525693e-3          # fineStructure x 1e-3, src/constants.f90:47
T_NODES, T_WEIGHTS = np.polynomial.hermite.hermgauss(40)
X = sp.Symbol("x", real=True)


def _gauss_1d(center, alpha, power, deriv):
    """Callable d^deriv/dx^deriv [(x - c)^p exp(-alpha (x - c)^2)]."""
    f = (X - center) ** power * sp.exp(-alpha * (X - center) ** 2)
    return sp.lambdify(X, sp.diff(f, X, deriv) if deriv else f, "numpy")


def _integral_1d(fa, fb, extra, z, P):
    """int fa(x) fb(x) extra(x) dx over the product Gaussian centred at P with
    exponent z, by Gauss-Hermite quadrature (the Gaussians are inside f)."""
    x = P + T_NODES / math.sqrt(z)
    vals = fa(x) * fb(x) * extra(x) * np.exp(T_NODES ** 2)
    return float(np.sum(T_WEIGHTS * vals) / math.sqrt(z))


def _block(kind, a1, a2, a3, A, B, C, l1, l2):
    """sh(l1 x l2) by quadrature.  kind 1 overlap, 2 kinetic, 4 three-centre
    overlap with exp(-a3 |r - C|^2), 5 mass velocity."""
    z = a1 + a2 + (a3 if kind == 4 else 0.0)
    out = np.zeros((l1, l2))
    cache = {}

    def one_d(d, ia, jb, deriv):
        key = (d, ia, jb, deriv)
        if key not in cache:
            fa = _gauss_1d(A[d], a1, ia, 0)
            fb = _gauss_1d(B[d], a2, jb, deriv)
            if kind == 4:
                extra = sp.lambdify(X, sp.exp(-a3 * (X - C[d]) ** 2), "numpy")
                P = (a1 * A[d] + a2 * B[d] + a3 * C[d]) / z
            else:
                extra = lambda x: np.ones_like(x)
                P = (a1 * A[d] + a2 * B[d]) / z
            cache[key] = _integral_1d(fa, fb, extra, z, P)
        return cache[key]

    def cart(ea, eb):
        if kind in (1, 4):
            return np.prod([one_d(d, ea[d], eb[d], 0) for d in range(3)])
        i0 = [one_d(d, ea[d], eb[d], 0) for d in range(3)]
        i2 = [one_d(d, ea[d], eb[d], 2) for d in range(3)]
        if kind == 2:                           # -1/2 nabla^2
            return -0.5 * (i2[0] * i0[1] * i0[2] + i0[0] * i2[1] * i0[2] + i0[0] * i0[1] * i2[2])
        i4 = [one_d(d, ea[d], eb[d], 4) for d in range(3)]
        lap2 = (i4[0] * i0[1] * i0[2] + i0[0] * i4[1] * i0[2] + i0[0] * i0[1] * i4[2]
                + 2 * (i2[0] * i2[1] * i0[2] + i2[0] * i0[1] * i2[2] + i0[0] * i2[1] * i2[2]))
        return FINE ** 2 / 8.0 * lap2

    for p in range(l1):
        for q in range(l2):
            out[p, q] = sum(ca * cb * cart(ea, eb) for ca, ea in HARM[p] for cb, eb in HARM[q])
    return out


def _tol(kind, ref, a1, a2, A, B, l1, l2, scale=None):
    """1e-10 of the block; for the mass velocity also 16 ulp of its
    expansion's absolute scale, which the nabla^4 terms cancel down from
    (by up to six orders for an f function on a steep exponent)."""
    tol = 1e-10 * np.abs(ref).max()
    if kind == 5:
        lof = {1: 0, 4: 1, 9: 2, 16: 3}
        if scale is None:
            scale = orc.massvel_scale(a1, a2, A, B, lof[l1], lof[l2])
        tol += 16 * 2.0 ** -52 * scale
    return tol


@pytest.mark.parametrize("kind", [1, 2, 4, 5])
def test_primitives_match_quadrature(kind):
    rng = np.random.default_rng(100 + kind)
    for l1, l2 in [(1, 1), (4, 1), (1, 9), (4, 4), (9, 4), (9, 9), (16, 4), (9, 16)]:
        a1, a2, a3 = np.exp(rng.uniform(np.log(0.15), np.log(20.0), 3))
        A, B, C = rng.uniform(-1.0, 1.0, (3, 3))
        got = orc.primitive(kind, [a1, a2, a3, *A, *B, *C], [l1, l2])[:l1, :l2]
        ref = _block(kind, a1, a2, a3, A, B, C, l1, l2)
        assert np.abs(got - ref).max() <= _tol(kind, ref, a1, a2, A, B, l1, l2), (kind, l1, l2)


def test_reference_goldens_match_quadrature(golden):
    """A sample of the reference's own blocks (two-centre and three-centre
    overlaps, kinetic, mass velocity) by quadrature, moderate exponents."""
    checked = 0
    for i in range(len(golden["kind"])):
        k = int(golden["kind"][i])
        p = golden["params"][i]
        if k == 3 or max(p[0], p[1], p[2]) > 100.0 or i % 5:
            continue
        l1, l2 = (int(x) for x in golden["lmalpha"][i])
        ref = _block(k, p[0], p[1], p[2], p[3:6], p[6:9], p[9:12], l1, l2)
        gold = golden["sh"][i][:l1, :l2]
        tol = _tol(k, ref, p[0], p[1], p[3:6], p[6:9], l1, l2, scale=golden["scale"][i])
        assert np.abs(gold - ref).max() <= tol, (i, k, l1, l2)
        checked += 1
    assert checked >= 40
