"""Raw layout-identical writers of the reference's HDF5 datasets.

Dataset names, dims and element order follow hdf5SetupIntg.F90:86-222
(integrals: (2, n(n+1)/2) per k and term) and hdf5MainEval.f90:60-81 /
hdf5MainEvec.F90:81-119 (eigenvalues (numStates) and eigenvectors
(valeDim, numStates) as separate real and imaginary datasets per k, spin).
"""

import json
import os

import numpy as np
import pytest

import oracle as orc
from olcao_gb300 import system as S


def test_eigen_writer_layout(tmp_path, gpu_free_lib):
    from olcao_gb300 import api
    rng = np.random.default_rng(5)
    nk, ns, nv = 3, 4, 6
    ev = np.sort(rng.normal(size=(nk, ns)), axis=1)
    vec = rng.normal(size=(nk, ns, nv)) + 1j * rng.normal(size=(nk, ns, nv))
    root = str(tmp_path / "main-temp")
    api.write_eigen(root, ev, vec, spin=2)
    man = json.load(open(os.path.join(root, "manifest.json")))
    paths = [d["path"] for d in man["datasets"]]
    assert paths[:3] == ["/eigenValues/00000010000002", "/eigenVectors/real00000010000002",
                         "/eigenVectors/imag00000010000002"]
    assert len(paths) == 3 * nk
    for k in range(nk):
        name = f"{k + 1:07d}{2:07d}"
        w = api.read_dataset(root, "/eigenValues/" + name)
        assert w.shape == (ns,) and np.array_equal(w, ev[k])
        re = api.read_dataset(root, "/eigenVectors/real" + name)
        im = api.read_dataset(root, "/eigenVectors/imag" + name)
        # (valeDim, numStates): column s is eigenvector s
        assert re.shape == (nv, ns)
        assert np.array_equal(re, vec[k].real.T) and np.array_equal(im, vec[k].imag.T)
        raw = np.fromfile(os.path.join(root, "eigenVectors", "real" + name + ".bin"), "<f8")
        assert np.array_equal(raw, vec[k].real.reshape(-1))   # Fortran order on disk


def test_eigen_writer_rejects_bad_sizes(tmp_path, gpu_free_lib):
    from olcao_gb300 import api
    with pytest.raises(api.OlcError):
        api.write_eigen(str(tmp_path / "x"), np.zeros((2, 5)), np.zeros((2, 5, 3)))


@pytest.mark.gpu
def test_setup_integrals_layout_matches_oracle(tmp_path, gpu_lib):
    from olcao_gb300 import api
    sysm = S.small_test_system("si2", nk=(2, 1, 1))
    o = orc.Oracle(sysm)
    packed = o.packed_operators()
    ctx = api.Context(sysm)
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
    root = str(tmp_path / "setup-temp")
    ctx.write_setup_integrals(root)
    plen = o.vale_dim * (o.vale_dim + 1) // 2
    names = {"atomOverlap": "S", "atomKEOverlap": "KE", "atomNucOverlap": "NP"}
    for k in range(o.nk):
        kn = f"{k + 1:07d}"
        for grp, key in names.items():
            d = api.read_dataset(root, f"/atomIntgGroup/{grp}/{kn}")
            assert d.shape == (2, plen)
            ref = packed[key][k].T          # oracle: [plen, (re, im)]
            assert np.abs(d - ref).max() <= 1e-10 * np.abs(ref).max() + 1e-14, (grp, k)
        for j in range(o.pot_dim):
            d = api.read_dataset(root, f"/atomIntgGroup/atomPotOverlap/{kn}/{j + 1:07d}")
            ref = packed[f"V{j}"][k].T
            assert np.abs(d - ref).max() <= 1e-10 * np.abs(ref).max() + 1e-14, (j, k)
