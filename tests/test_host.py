"""Host-side logic and the C ABI (no GPU needed)."""

import ctypes
import os
import re

import numpy as np
import pytest

from olcao_gb300 import system as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "olcao_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(olc_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from olcao_gb300 import api, build
    if not os.path.exists(api.LIB_PATH):
        build.build()
    lib = ctypes.CDLL(api.LIB_PATH)
    names = _declared_functions()
    assert len(names) >= 13
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/olcao_gpu.h but not exported"
    assert set(api.EXPORTS) <= set(names)
    assert api.lib().olc_version().startswith(b"olcao_gb300")


def test_library_rejects_bad_arguments_without_gpu():
    from olcao_gb300 import api
    L = api.lib()
    assert L.olc_create(None, None, None) != 0
    assert L.olc_primitive_batch(9, 1, None, None, None) != 0
    # g-type (l = 4) exponents are outside the kernels and report it
    out = np.zeros(256)
    p = np.zeros(12)
    lm = np.array([25, 1], np.int32)
    st = L.olc_primitive_batch(1, 1, p.ctypes.data, lm.ctypes.data, out.ctypes.data)
    assert st == 1 and "lmalpha" in api.last_error()


@pytest.mark.parametrize("name,nv,nc,nk", [
    ("diamond", 10, 2, 216), ("si64", 832, 320, 64), ("graphite", 32, 0, 8192),
    ("si8", 104, 0, 512), ("quartz", 3159, 567, 9), ("si512", 6656, 2560, 9)])
def test_synthetic_configs_have_the_stated_sizes(name, nv, nc, nk):
    s = S.SYSTEMS[name]()
    assert (s.vale_dim, s.core_dim, s.num_kpoints) == (nv, nc, nk)
    assert np.isclose(s.kpoint_weights().sum(), 2.0)
    # atoms do not collide
    d = s.site_pos[:, None, :] - s.site_pos[None, :, :]
    r = np.sqrt((d ** 2).sum(-1)) + np.eye(len(s.site_pos)) * 1e9
    assert r.min() > 1.5


def test_radial_functions_are_normalised():
    s = S.silicon_supercell(1, 0.0, seed=3, mesh=(1, 1, 1))
    t = s.types[0]
    for r, l in enumerate(t.vale_l):
        n = t.num_orb_alphas[l]
        assert np.isclose(S.radial_norm(t.vale_coeff[r, :n], t.alphas[:n], l), 1.0)


def test_kpoint_mesh_matches_reference_formula():
    kp = S.mp_mesh((2, 2, 2), (0.5, 0.5, 0.5))
    assert np.allclose(np.unique(kp), [-0.25, 0.25])
    kp0 = S.mp_mesh((3, 1, 1))
    assert np.allclose(kp0[:, 0], [-0.5, -0.5 + 1 / 3, -0.5 + 2 / 3])


def test_reference_assembly_rule():
    import oracle as orc
    packed = {"NP": np.ones((1, 3, 2)), "KE": np.ones((1, 3, 2)),
              "V0": np.ones((1, 3, 2)), "V1": np.ones((1, 3, 2))}
    h = orc.assemble(packed, np.array([0.0, 2.0]))
    assert np.allclose(h, 1 + 1 + 1 + 2)      # zero multiplier adds unscaled


def test_g_functions_are_refused_by_the_gpu_build(gpu_free_lib):
    """The device kernels are built for s, p, d, f; a radial function with
    l = 4 is refused with OLC_ERR_ARG before any device work."""
    from olcao_gb300 import api
    with pytest.raises(api.OlcError) as e:
        api.primitive_batch(1, np.zeros((1, 12)) + 1.0, np.array([[25, 1]], np.int32))
    assert e.value.status == 1


def test_fortran_binding_covers_every_entry_point():
    """include/olcao_gpu.f90 (the ISO_C_BINDING module a maintainer adds to
    the reference's build) binds every entry point include/olcao_gpu.h
    declares, by the same name."""
    import os
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(root, "include", "olcao_gpu.h")) as fh:
        declared = set(re.findall(r"^(?:int|int64_t|const char\*)\s+(olc_\w+)\s*\(", fh.read(), re.M))
    with open(os.path.join(root, "include", "olcao_gpu.f90")) as fh:
        bound = set(re.findall(r'bind\s*\(\s*C\s*,\s*name\s*=\s*"(olc_\w+)"', fh.read(), re.I))
    assert declared and declared == bound, (sorted(declared - bound), sorted(bound - declared))
