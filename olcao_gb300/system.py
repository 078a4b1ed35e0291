"""System description (ctypes mirror of ``olc_system_t``) and the seeded
synthetic structures the hot path is measured and tested on.

The reference reads these inputs from its ``olcao.dat``/``structure.dat``
files (src/olcao/input.f90:114-231, atomicTypes.f90, potTypes.f90,
atomicSites.f90, potSites.f90, kpoints.f90).  No such input set ships with
the reference for the five structures of interest, so they are generated
here with fixed seeds:

* even-tempered exponents  alpha_i = min * (max/min)**((i-1)/(N-1))
  (the formula of makePotAlphas, src/olcao/potTypes.f90:187-192);
* radial contraction coefficients ~ N(0, 1), rescaled so that each radial
  function has unit norm over its own Gaussians;
* potential coefficients ~ 0.1 * N(0, 1);
* Gaussian displacements of the atoms with the stated sigma;
* Monkhorst-Pack meshes k = -1/2 + (i - 1 + shift)/n per axis
  (src/uolcao/kpoints.f90:770-783), no symmetry reduction.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Dict, List, Sequence, Tuple

import numpy as np

ANGSTROM = 1.0 / 0.529177210903   # bohr per angstrom (src/constants.f90)
MAX_ALPHAS = 32
MAX_RADIAL = 12
MAX_POT_ALPHAS = 32


class AtomType(C.Structure):
    _fields_ = [("element", C.c_int32),
                ("num_orb_alphas", C.c_int32 * 4),
                ("alphas", C.c_double * MAX_ALPHAS),
                ("num_vale_radial", C.c_int32),
                ("num_core_radial", C.c_int32),
                ("radial_l", C.c_int32 * MAX_RADIAL),
                ("radial_coeff", (C.c_double * MAX_ALPHAS) * MAX_RADIAL)]


class PotType(C.Structure):
    _fields_ = [("element", C.c_int32),
                ("num_alphas", C.c_int32),
                ("nuc_charge", C.c_double),
                ("nuc_alpha", C.c_double),
                ("alphas", C.c_double * MAX_POT_ALPHAS)]


class SystemStruct(C.Structure):
    _fields_ = [("real_vectors", C.c_double * 9),
                ("num_atom_types", C.c_int32),
                ("atom_types", C.POINTER(AtomType)),
                ("num_atom_sites", C.c_int32),
                ("site_type", C.POINTER(C.c_int32)),
                ("site_pos", C.POINTER(C.c_double)),
                ("num_pot_types", C.c_int32),
                ("pot_types", C.POINTER(PotType)),
                ("num_pot_sites", C.c_int32),
                ("pot_site_type", C.POINTER(C.c_int32)),
                ("pot_site_pos", C.POINTER(C.c_double)),
                ("num_kpoints", C.c_int32),
                ("kpoints_abc", C.POINTER(C.c_double)),
                ("basis_fn_thresh", C.c_double),
                ("rel", C.c_int32)]


@dataclass
class TypeSpec:
    element: int
    alphas: np.ndarray                 # ascending
    num_orb_alphas: Tuple[int, int, int, int]
    vale_l: List[int]
    core_l: List[int]
    vale_coeff: np.ndarray = None      # [nvale, nalpha]
    core_coeff: np.ndarray = None      # [ncore, nalpha]

    @property
    def num_vale_states(self) -> int:
        return sum(2 * l + 1 for l in self.vale_l)

    @property
    def num_core_states(self) -> int:
        return sum(2 * l + 1 for l in self.core_l)


@dataclass
class PotSpec:
    element: int
    nuc_charge: float
    nuc_alpha: float
    alphas: np.ndarray


@dataclass
class System:
    """A complete, seeded input set for the hot path."""
    name: str
    real_vectors: np.ndarray           # [3, 3], column = a, b, c (bohr)
    types: List[TypeSpec]
    site_type: np.ndarray              # [n] 0-based
    site_pos: np.ndarray               # [n, 3] bohr
    pots: List[PotSpec]
    pot_site_type: np.ndarray
    pot_site_pos: np.ndarray
    kpoints_abc: np.ndarray            # [nk, 3]
    pot_coeffs: np.ndarray             # [pot_dim]
    thresh: float = 1e-16
    seed: int = 0
    rel: int = 0                       # 1: scalar relativistic (mass-velocity term)
    _keep: list = field(default_factory=list, repr=False)

    # ---- derived sizes -------------------------------------------------
    @property
    def vale_dim(self) -> int:
        return int(sum(self.types[t].num_vale_states for t in self.site_type))

    @property
    def core_dim(self) -> int:
        return int(sum(self.types[t].num_core_states for t in self.site_type))

    @property
    def pot_dim(self) -> int:
        return int(sum(len(p.alphas) for p in self.pots))

    @property
    def num_kpoints(self) -> int:
        return int(self.kpoints_abc.shape[0])

    def kpoint_weights(self) -> np.ndarray:
        """Weight 2/N per k (spin-degenerate), src/uolcao/kpoints.f90:804-810."""
        return np.full(self.num_kpoints, 2.0 / self.num_kpoints)

    # ---- ctypes view -----------------------------------------------------
    def to_struct(self) -> SystemStruct:
        at = (AtomType * len(self.types))()
        for i, t in enumerate(self.types):
            r = at[i]
            r.element = t.element
            for l in range(4):
                r.num_orb_alphas[l] = t.num_orb_alphas[l]
            for a, v in enumerate(t.alphas):
                r.alphas[a] = float(v)
            r.num_vale_radial = len(t.vale_l)
            r.num_core_radial = len(t.core_l)
            for k, l in enumerate(list(t.vale_l) + list(t.core_l)):
                r.radial_l[k] = l
            coeffs = list(t.vale_coeff) + list(t.core_coeff)
            for k, c in enumerate(coeffs):
                for a, v in enumerate(c):
                    r.radial_coeff[k][a] = float(v)
        pt = (PotType * len(self.pots))()
        for i, p in enumerate(self.pots):
            pt[i].element = p.element
            pt[i].num_alphas = len(p.alphas)
            pt[i].nuc_charge = p.nuc_charge
            pt[i].nuc_alpha = p.nuc_alpha
            for a, v in enumerate(p.alphas):
                pt[i].alphas[a] = float(v)
        arrs = dict(
            site_type=np.ascontiguousarray(self.site_type, np.int32),
            site_pos=np.ascontiguousarray(self.site_pos, np.float64),
            pot_site_type=np.ascontiguousarray(self.pot_site_type, np.int32),
            pot_site_pos=np.ascontiguousarray(self.pot_site_pos, np.float64),
            kp=np.ascontiguousarray(self.kpoints_abc, np.float64))
        s = SystemStruct()
        for i in range(3):
            for j in range(3):
                s.real_vectors[j * 3 + i] = float(self.real_vectors[i, j])
        s.num_atom_types = len(self.types)
        s.atom_types = C.cast(at, C.POINTER(AtomType))
        s.num_atom_sites = len(self.site_type)
        s.site_type = arrs["site_type"].ctypes.data_as(C.POINTER(C.c_int32))
        s.site_pos = arrs["site_pos"].ctypes.data_as(C.POINTER(C.c_double))
        s.num_pot_types = len(self.pots)
        s.pot_types = C.cast(pt, C.POINTER(PotType))
        s.num_pot_sites = len(self.pot_site_type)
        s.pot_site_type = arrs["pot_site_type"].ctypes.data_as(C.POINTER(C.c_int32))
        s.pot_site_pos = arrs["pot_site_pos"].ctypes.data_as(C.POINTER(C.c_double))
        s.num_kpoints = self.num_kpoints
        s.kpoints_abc = arrs["kp"].ctypes.data_as(C.POINTER(C.c_double))
        s.basis_fn_thresh = self.thresh
        s.rel = int(self.rel)
        self._keep[:] = [at, pt, arrs]
        return s


# ---------------------------------------------------------------------------
# builders
# ---------------------------------------------------------------------------

def even_tempered(n: int, amin: float, amax: float) -> np.ndarray:
    r = (amax / amin) ** (1.0 / (n - 1))
    return np.array([amin * r ** i for i in range(n)])


def radial_norm(coeff: np.ndarray, alphas: np.ndarray, l: int) -> float:
    """Norm of R(r) = sum_i c_i r^l exp(-a_i r^2) times a unit harmonic."""
    s = alphas[:, None] + alphas[None, :]
    g = math.gamma(l + 1.5) / (2.0 * s ** (l + 1.5))
    return float(np.sqrt(coeff @ g @ coeff))


def _radials(rng, alphas, orb, ls) -> np.ndarray:
    out = np.zeros((len(ls), len(alphas)))
    for k, l in enumerate(ls):
        n = orb[l]
        c = rng.standard_normal(n)
        c /= radial_norm(c, alphas[:n], l)
        out[k, :n] = c
    return out


def make_type(rng, element, nalpha, amin, amax, orb, vale_l, core_l) -> TypeSpec:
    al = even_tempered(nalpha, amin, amax)
    t = TypeSpec(element=element, alphas=al, num_orb_alphas=tuple(orb),
                 vale_l=list(vale_l), core_l=list(core_l))
    t.vale_coeff = _radials(rng, al, orb, vale_l)
    t.core_coeff = _radials(rng, al, orb, core_l)
    return t


def mp_mesh(n: Sequence[int], shift=(0.0, 0.0, 0.0)) -> np.ndarray:
    pts = []
    for i in range(1, n[0] + 1):
        for j in range(1, n[1] + 1):
            for k in range(1, n[2] + 1):
                idx = np.array([i, j, k], float)
                pts.append(-0.5 + (idx - 1.0 + np.asarray(shift)) / np.asarray(n, float))
    return np.array(pts)


def gamma_plus_shifted_222() -> np.ndarray:
    return np.vstack([np.zeros((1, 3)), mp_mesh((2, 2, 2), (0.5, 0.5, 0.5))])


def _supercell(prim_vec, frac, reps):
    """prim_vec [3,3] columns; frac [n,3] fractional in prim cell."""
    pos = []
    for i in range(reps[0]):
        for j in range(reps[1]):
            for k in range(reps[2]):
                for f in frac:
                    pos.append(prim_vec @ (np.asarray(f) + [i, j, k]))
    vec = prim_vec * np.asarray(reps)[None, :]
    return vec, np.array(pos)


def _finish(name, vec, types, site_type, pos, pots, kp, rng, seed,
            sigma_ang=0.0, pot_of_type=None):
    if sigma_ang > 0:
        pos = pos + rng.normal(0.0, sigma_ang * ANGSTROM, size=pos.shape)
    site_type = np.asarray(site_type, np.int32)
    # potential sites: one per atom, grouped by potential type
    ptype = np.array([pot_of_type[t] for t in site_type], np.int32)
    order = np.argsort(ptype, kind="stable")
    pot_coeffs = 0.1 * rng.standard_normal(sum(len(p.alphas) for p in pots))
    return System(name=name, real_vectors=vec, types=types, site_type=site_type,
                  site_pos=pos, pots=pots, pot_site_type=ptype[order],
                  pot_site_pos=pos[order], kpoints_abc=kp,
                  pot_coeffs=pot_coeffs, seed=seed)


def carbon_type(rng, vale_l=(0, 1, 0), core_l=(0,)) -> TypeSpec:
    return make_type(rng, 1, 16, 0.15, 5.0e4, (16, 16, 0, 0), vale_l, core_l)


def carbon_pot(element=1) -> PotSpec:
    return PotSpec(element, 6.0, 20.0, even_tempered(12, 0.1, 1.0e5))


def silicon_type(rng, element=1, core=True) -> TypeSpec:
    return make_type(rng, element, 18, 0.12, 1.0e6, (18, 18, 12, 0),
                     (0, 1, 2, 0, 1), (0, 0, 1) if core else ())


def silicon_pot(element=1) -> PotSpec:
    return PotSpec(element, 14.0, 20.0, even_tempered(16, 0.1, 1.0e6))


def diamond(seed: int = 1, mesh=(6, 6, 6)) -> System:
    """Config 1: 2-atom FCC diamond, a = 3.567 A, 216 k (6x6x6 MP)."""
    rng = np.random.default_rng(seed)
    a = 3.567 * ANGSTROM
    vec = 0.5 * a * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], float).T
    pos = np.array([[0, 0, 0], [0.25 * a] * 3])
    t = carbon_type(rng)
    return _finish("diamond", vec, [t], [0, 0], pos, [carbon_pot()],
                   mp_mesh(mesh), rng, seed, pot_of_type={0: 0})


def silicon_supercell(reps=2, sigma=0.03, seed: int = 2, mesh=(4, 4, 4),
                      core=True, kp=None, name=None) -> System:
    """Config 2 (reps=2) / config 5 (reps=4): conventional diamond Si."""
    rng = np.random.default_rng(seed)
    a = 5.431 * ANGSTROM
    frac8 = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                      [.25, .25, .25], [.25, .75, .75], [.75, .25, .75],
                      [.75, .75, .25]])
    vec, pos = _supercell(a * np.eye(3), frac8, (reps,) * 3)
    t = silicon_type(rng, core=core)
    kpts = mp_mesh(mesh) if kp is None else kp
    return _finish(name or f"si{8 * reps ** 3}", vec, [t], [0] * len(pos), pos,
                   [silicon_pot()], kpts, rng, seed, sigma_ang=sigma,
                   pot_of_type={0: 0})


def graphite(seed: int = 3, mesh=(32, 32, 8)) -> System:
    """Config 3a: AB graphite, 4 atoms, C 2s2p3s3p valence only (n = 32)."""
    rng = np.random.default_rng(seed)
    a, c = 2.46 * ANGSTROM, 6.71 * ANGSTROM
    vec = np.array([[a, 0, 0], [-0.5 * a, 0.5 * math.sqrt(3) * a, 0],
                    [0, 0, c]]).T
    frac = np.array([[0, 0, .25], [0, 0, .75], [1 / 3, 2 / 3, .25],
                     [2 / 3, 1 / 3, .75]])
    pos = frac @ vec.T
    t = carbon_type(rng, vale_l=(0, 1, 0, 1), core_l=())
    return _finish("graphite", vec, [t], [0] * 4, pos, [carbon_pot()],
                   mp_mesh(mesh), rng, seed, pot_of_type={0: 0})


def quartz(seed: int = 4, reps=3, sigma=0.05) -> System:
    """Config 4: alpha-quartz SiO2 3x3x3 (243 atoms), Gamma + 2x2x2."""
    rng = np.random.default_rng(seed)
    a, c = 4.913 * ANGSTROM, 5.405 * ANGSTROM
    pvec = np.array([[a, 0, 0], [-0.5 * a, 0.5 * math.sqrt(3) * a, 0],
                     [0, 0, c]]).T
    u, x, y, z = 0.47, 0.41, 0.27, 0.12
    si = [[u, 0, 1 / 3], [0, u, 2 / 3], [-u, -u, 0]]
    ox = [[x, y, z], [-y, x - y, z + 1 / 3], [y - x, -x, z + 2 / 3],
          [y, x, -z], [x - y, -y, 2 / 3 - z], [-x, y - x, 1 / 3 - z]]
    frac = np.mod(np.array(si + ox), 1.0)
    vec, pos = _supercell(pvec, frac, (reps,) * 3)
    kinds = ([0] * 3 + [1] * 6) * reps ** 3
    tsi = silicon_type(rng, element=1)
    to = make_type(rng, 2, 18, 0.12, 1.0e6, (18, 18, 12, 0),
                   (0, 1, 0, 1, 2), (0,))
    pots = [silicon_pot(1), PotSpec(2, 8.0, 20.0, even_tempered(16, 0.1, 1.0e6))]
    return _finish("quartz", vec, [tsi, to], kinds, pos, pots,
                   gamma_plus_shifted_222(), rng, seed, sigma_ang=sigma,
                   pot_of_type={0: 0, 1: 1})


SYSTEMS = {
    "diamond": lambda: diamond(),
    "si64": lambda: silicon_supercell(2, 0.03, seed=2),
    "graphite": lambda: graphite(),
    "si8": lambda: silicon_supercell(1, 0.0, seed=5, mesh=(8, 8, 8),
                                     core=False, name="si8"),
    "quartz": lambda: quartz(),
    "si512": lambda: silicon_supercell(4, 0.05, seed=6,
                                       kp=gamma_plus_shifted_222(),
                                       name="si512"),
}


def small_test_system(kind: str = "si2", seed: int = 11, nk=(2, 2, 2)) -> System:
    """Tiny seeded systems the CPU oracle finishes in seconds.

    si2: 2 Si atoms in a small triclinic-ish cell with core states and d
    functions; c2: diamond primitive cell with a coarse mesh; sio: one Si
    and one O (two types, two potential types); sif: sio with f functions
    on Si (a valence f and a core f), so that every class pair s..f meets."""
    rng = np.random.default_rng(seed)
    if kind == "tiny":
        a = 3.567 * ANGSTROM
        vec = 0.5 * a * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], float).T
        pos = np.array([[0, 0, 0], [0.25 * a] * 3])
        t = make_type(rng, 1, 8, 0.5, 2.0e3, (8, 8, 5, 0), (0, 1, 2), (0,))
        pot = PotSpec(1, 6.0, 20.0, even_tempered(4, 0.4, 1.0e3))
        return _finish("tiny", vec, [t], [0, 0], pos, [pot],
                       mp_mesh(nk, (0.5, 0.5, 0.5)), rng, seed, sigma_ang=0.02,
                       pot_of_type={0: 0})
    if kind == "c2":
        return diamond(seed=seed, mesh=nk)
    if kind == "si2":
        a = 5.431 * ANGSTROM
        vec = 0.5 * a * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], float).T
        pos = np.array([[0, 0, 0], [0.25 * a] * 3])
        t = silicon_type(rng)
        return _finish("si2", vec, [t], [0, 0], pos, [silicon_pot()],
                       mp_mesh(nk, (0.5, 0.5, 0.5)), rng, seed, sigma_ang=0.02,
                       pot_of_type={0: 0})
    if kind == "sio":
        a = 4.0 * ANGSTROM
        vec = np.array([[a, 0, 0], [0.2 * a, 0.95 * a, 0], [0.1 * a, 0.15 * a, 1.1 * a]]).T
        pos = np.array([[0.1, 0.2, 0.3], [1.5, 1.2, 1.9]]) * ANGSTROM
        tsi = silicon_type(rng, element=1)
        to = make_type(rng, 2, 18, 0.12, 1.0e6, (18, 18, 12, 0),
                       (0, 1, 0, 1, 2), (0,))
        pots = [silicon_pot(1), PotSpec(2, 8.0, 20.0, even_tempered(16, 0.1, 1.0e6))]
        return _finish("sio", vec, [tsi, to], [0, 1], pos, pots,
                       mp_mesh(nk, (0.5, 0.5, 0.5)), rng, seed,
                       pot_of_type={0: 0, 1: 1})
    if kind == "sif":
        a = 4.2 * ANGSTROM
        vec = np.array([[a, 0, 0], [0.1 * a, a, 0], [0.2 * a, 0.1 * a, 1.05 * a]]).T
        pos = np.array([[0.1, 0.2, 0.3], [1.4, 1.3, 1.8]]) * ANGSTROM
        tsi = make_type(rng, 1, 18, 0.12, 1.0e6, (18, 18, 12, 8),
                        (0, 1, 2, 3, 0, 1), (0, 0, 1, 3))
        to = make_type(rng, 2, 18, 0.12, 1.0e6, (18, 18, 12, 0),
                       (0, 1, 0, 1, 2), (0,))
        pots = [silicon_pot(1), PotSpec(2, 8.0, 20.0, even_tempered(16, 0.1, 1.0e6))]
        return _finish("sif", vec, [tsi, to], [0, 1], pos, pots,
                       mp_mesh(nk, (0.5, 0.5, 0.5)), rng, seed,
                       pot_of_type={0: 0, 1: 1})
    raise ValueError(kind)
