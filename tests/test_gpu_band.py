"""Band structure on a k-point path (the reference's band program,
src/olcao/OLCAO_Band.F90:109-255) through the GPU library (gpu).

A two-atom system with core states and d functions on two paths through
high-symmetry points: the stored form's eigenvalues against LAPACK zhegv on
the oracle's H(k), S(k) at the same path k-points (1e-8 Ha), and the fused
form (the band program's recomputed integrals) against the stored form
(1e-6 Ha: the fused form flushes small values once per summed operator, the
reference's storage form once per stored term)."""

import dataclasses

import numpy as np
import pytest

import oracle as orc
from olcao_gb300 import band
from olcao_gb300 import system as S

EIG_TOL = 1e-8

PATHS = [np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.5, 0.5, 0.0]]),
         np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])]


@pytest.mark.gpu
def test_band_structure_matches_oracle_on_the_path(gpu_lib):
    from olcao_gb300 import api
    sysm = S.small_test_system("si2", nk=(1, 1, 1))
    w, mag, k_cart = band.band_structure(sysm, PATHS, 9, form=api.FORM_STORED)
    nk = len(mag)
    assert w.shape == (nk, sysm.vale_dim) and np.all(np.diff(mag) >= 0)
    part = dataclasses.replace(sysm, kpoints_abc=band.to_fractional(sysm.real_vectors, k_cart), _keep=[])
    o = orc.Oracle(part)
    packed = o.packed_operators()
    ref, _ = orc.zhegv(orc.assemble(packed, sysm.pot_coeffs), packed["S"], o.vale_dim, o.vale_dim)
    assert np.abs(w - ref).max() <= EIG_TOL
    wf, magf, _ = band.band_structure(sysm, PATHS, 9)
    assert np.allclose(magf, mag)
    assert np.abs(wf - w).max() <= 1e-6
