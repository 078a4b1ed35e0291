"""Band structure along a path of k-points through the GPU library.

The reference's band program (OLCAO_Band, src/olcao/OLCAO_Band.F90:24-255)
replaces the SCF mesh by a path through high-symmetry k-points
(makePathKPoints, src/olcao/kpoints.f90:313-534), recomputes the integrals
on that path with the converged potential and solves one generalised
eigen-problem per k (computeBands -> getIntgResults, secularEqnOneKP).  Here
the path is built on the host exactly as makePathKPoints builds it, and the
integrals, orthogonalisation, Hamiltonian and solves run on the GPU for all
path k-points at once (olc_create, olc_scf_prepare, olc_scf_iteration).
"""

from __future__ import annotations

import dataclasses
import math
from typing import List, Sequence, Tuple

import numpy as np


def recip_vectors(real_vectors: np.ndarray) -> np.ndarray:
    """Reciprocal lattice vectors as rows, b_i = 2 pi (a_j x a_k) / V, from
    the real vectors given as columns (the library's lattice convention,
    src/olcao/lattice.f90)."""
    a = [np.asarray(real_vectors, float)[:, i] for i in range(3)]
    vol = float(np.dot(a[0], np.cross(a[1], a[2])))
    if abs(vol) < 1e-12:
        raise ValueError("singular lattice")
    return np.array([2.0 * math.pi * np.cross(a[(i + 1) % 3], a[(i + 2) % 3]) / vol for i in range(3)])


def to_fractional(real_vectors: np.ndarray, k_cart: np.ndarray) -> np.ndarray:
    """Cartesian k-points [nk, 3] as fractions of the reciprocal vectors (the
    library's kpoints_abc), the inverse of k = sum_i abc_i b_i."""
    return np.asarray(k_cart, float) @ np.linalg.inv(recip_vectors(real_vectors))


def path_kpoints(real_vectors: np.ndarray, paths: Sequence[np.ndarray], num_path_kp: int,
                 cartesian: bool = False) -> Tuple[np.ndarray, np.ndarray, np.ndarray, List[int]]:
    """makePathKPoints (src/olcao/kpoints.f90:313-534).

    paths: one array [m_i, 3] of high-symmetry points per path, fractional
    coordinates of the reciprocal cell unless `cartesian`.  A new path starts
    at the distance where the previous one ended.  When num_path_kp equals
    the number of high-symmetry points, those points are the path; otherwise
    the average spacing is the path's length / (num_path_kp - 1) and each
    segment gets int(length / spacing) steps (fewer if that would pass
    num_path_kp), its interior points at equal Cartesian steps, followed by
    the segment's end point.  A segment with no step keeps the previous
    segment's step for the magnitude of its end point, as the reference
    does.

    Returns (k-points in Cartesian coordinates [nk, 3], the distance along
    the path of each point [nk], the weights 2 / nk [nk], the 1-based
    indices of the high-symmetry points in the list).
    """
    if num_path_kp < 1:
        raise ValueError("num_path_kp must be positive")
    B = recip_vectors(real_vectors)
    hs = [np.asarray(p, float).reshape(-1, 3) for p in paths]
    if not hs or any(len(p) == 0 for p in hs):
        raise ValueError("every path needs at least one high-symmetry point")
    if not cartesian:
        hs = [p @ B for p in hs]
    # distances between consecutive high-symmetry points (:380-403)
    dvec = [np.zeros_like(p) for p in hs]
    dmag = [np.zeros(len(p)) for p in hs]
    for i, p in enumerate(hs):
        for j in range(len(p)):
            if i == 0 and j == 0:
                continue
            if j == 0:
                dvec[i][0] = dvec[i - 1][-1]
                dmag[i][0] = dmag[i - 1][-1]
            else:
                dvec[i][j] = p[j] - p[j - 1]
                dmag[i][j] = dmag[i][j - 1] + math.sqrt(float(np.sum(dvec[i][j] ** 2)))
    kp: List[np.ndarray] = []
    mag: List[float] = []
    hs_index: List[int] = []
    if num_path_kp == sum(len(p) for p in hs):
        for i, p in enumerate(hs):
            for j in range(len(p)):
                kp.append(p[j])
                mag.append(float(dmag[i][j]))
                hs_index.append(len(kp))
    else:
        if num_path_kp < 2:
            raise ValueError("a path of interpolated points needs num_path_kp >= 2")
        avg = dmag[-1][-1] / (num_path_kp - 1)
        step = np.zeros(3)
        for i, p in enumerate(hs):
            for j in range(len(p)):
                if j != 0:
                    nseg = int((dmag[i][j] - dmag[i][j - 1]) / avg) if avg > 0 else 0
                    if len(kp) + nseg > num_path_kp:
                        nseg = num_path_kp - len(kp)
                    if nseg >= 1:
                        step = dvec[i][j] / nseg
                        for _ in range(nseg - 1):
                            kp.append(kp[-1] + step)
                            mag.append(mag[-1] + math.sqrt(float(np.sum(step ** 2))))
                kp.append(p[j].copy())
                hs_index.append(len(kp))
                if i == 0 and j == 0:
                    mag.append(0.0)
                elif j == 0:
                    mag.append(mag[-1])
                else:
                    mag.append(mag[-1] + math.sqrt(float(np.sum(step ** 2))))
    nk = len(kp)
    return np.array(kp), np.array(mag), np.full(nk, 2.0 / nk), hs_index


def band_structure(system, paths: Sequence[np.ndarray], num_path_kp: int, coeffs=None,
                   num_states: int = 0, cartesian: bool = False, form=None, precision=None):
    """Eigenvalues [nk, num_states] (Hartree) along the path, with the path
    distances [nk] and Cartesian k-points [nk, 3].

    system: the converged system (its pot_coeffs are used unless `coeffs`
    is given); the path replaces its k-point mesh.  form: FORM_FUSED by
    default (the band program recomputes the integrals with the potential);
    precision: PREC_FP64 by default (zhegv per k, as secularEqnOneKP).
    """
    from . import api
    k_cart, mag, _, _ = path_kpoints(system.real_vectors, paths, num_path_kp, cartesian)
    sub = dataclasses.replace(system, kpoints_abc=to_fractional(system.real_vectors, k_cart), _keep=[])
    form = api.FORM_FUSED if form is None else form
    precision = api.PREC_FP64 if precision is None else precision
    ctx = api.Context(sub)
    try:
        ctx.scf_prepare(api.PREC_FP64, form)
        c = system.pot_coeffs if coeffs is None else np.asarray(coeffs, float)
        eig = ctx.scf_iteration(c, num_states or ctx.vale_dim, precision=precision)
    finally:
        ctx.close()
    return eig, mag, k_cart
