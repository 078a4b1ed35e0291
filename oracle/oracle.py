"""ctypes front end of the CPU oracle (oracle/olcao_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py as the checker, never by the product.

Besides the compiled restatement of the reference loops this module holds the
eigen-solve leg of the oracle: scipy's LAPACK ``zhegv`` (the routine
src/olcao/interfaces.F90:105 calls) on the unpacked H(k), S(k), and numpy
restatements of the steps after the solve: populateStates
(src/olcao/populate.F90:132-578, with the merge sort of sortSubs.f90:18-175)
and makeValenceRho (src/olcao/valeCharge.F90:172-395).

Parity pinning: primitives pinned by the reference's own generated code
(tests/golden); everything above them -- drivers, eigen-solve call,
occupations, density traces -- parity unpinned (no reference fixtures for
this path, reference not buildable here).
"""

from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from typing import Dict, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB: Optional[C.CDLL] = None

OP_OVERLAP, OP_KINETIC, OP_NUCLEAR, OP_ELECPOT, OP_MASSVEL = 1, 2, 3, 4, 5


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return os.path.join(_HERE, "_build", "liboracle.so")


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle.so")
        src = os.path.join(_HERE, "olcao_oracle.cpp")
        if (not os.path.exists(path)) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = C.CDLL(path)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_void_p]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_error.restype = C.c_char_p
        L.orc_dims.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_cells.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_operator.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_void_p]
        L.orc_operator.restype = C.c_int
        L.orc_ortho_pack.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 5
        L.orc_set_pairs.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_primitive.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_boys.argtypes = [C.c_double, C.c_void_p]
        _LIB = L
    return _LIB


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def primitive(kind: int, params: Sequence[float], lmalpha: Sequence[int]) -> np.ndarray:
    """One primitive sh(16,16) block (column-major in memory, returned [16,16]
    indexed [row, col])."""
    inp = np.ascontiguousarray(params, np.float64)
    lm = np.ascontiguousarray(lmalpha, np.int32)
    out = np.zeros(256)
    lib().orc_primitive(kind, _p(inp), _p(lm), _p(out))
    return out.reshape(16, 16).T


def boys(T: float) -> np.ndarray:
    F = np.zeros(7)
    lib().orc_boys(float(T), _p(F))
    return F


class Oracle:
    """One system set up on the CPU (lattice, basis, tables)."""

    def __init__(self, system):
        self.system = system
        self._struct = system.to_struct()
        h = lib().orc_create(C.byref(self._struct))
        if not h:
            raise RuntimeError(lib().orc_error().decode())
        self.h = h
        d = np.zeros(5, np.int32)
        lib().orc_dims(h, _p(d))
        self.vale_dim, self.core_dim, self.pot_dim, self.nk, self.ncells = map(int, d)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def cells(self) -> np.ndarray:
        out = np.zeros((self.ncells, 4))
        lib().orc_cells(self.h, _p(out))
        return out

    def operator(self, op: int, term: int = 0):
        """Un-orthogonalised (vv, cv, cc) complex arrays, shape [nk, cols, rows]
        in memory order of the reference's (rows, cols, nk) column-major."""
        nv, nc, nk = self.vale_dim, self.core_dim, self.nk
        vv = np.zeros((nk, nv, nv), np.complex128)
        cv = np.zeros((nk, nv, nc), np.complex128) if nc else None
        cc = np.zeros((nk, nc, nc), np.complex128) if nc else None
        st = lib().orc_operator(self.h, op, term, _p(vv), _p(cv), _p(cc))
        if st:
            raise RuntimeError(f"oracle status {st}: {lib().orc_error().decode()}")
        return vv, cv, cc

    def set_pairs(self, pairs=None):
        """Restrict the operator passes to the atom pairs (i, j) listed
        (0-based); None restores all pairs.  Blocks of other pairs stay zero."""
        if not pairs:
            lib().orc_set_pairs(self.h, 0, None)
            return
        ij = np.ascontiguousarray(np.asarray(pairs, np.int32).reshape(-1, 2))
        lib().orc_set_pairs(self.h, int(ij.shape[0]), _p(ij))

    def ortho_pack(self, is_overlap: bool, vv, cv, cc, scv) -> np.ndarray:
        nv, nk = self.vale_dim, self.nk
        packed = np.zeros((nk, nv * (nv + 1) // 2, 2))
        vv = vv.copy()
        lib().orc_ortho_pack(self.h, int(is_overlap), _p(vv), _p(cv), _p(cc),
                             _p(scv), _p(packed))
        return packed

    # ---- convenience: the reference's stored integrals ----------------------
    def packed_operators(self, terms: Optional[Sequence[int]] = None) -> Dict[str, np.ndarray]:
        """Packed, orthogonalised S, KE, NP and V_j as the reference's
        OLCAOsetup writes them (integrals.F90 ortho + pack)."""
        vvS, cvS, ccS = self.operator(OP_OVERLAP)
        out = {"S": self.ortho_pack(True, vvS, cvS, ccS, cvS)}
        ops = (("KE", OP_KINETIC), ("NP", OP_NUCLEAR))
        if getattr(self.system, "rel", 0):
            ops += (("MV", OP_MASSVEL),)      # gaussOverlapMV, OLCAO_Setup.f90:142-144
        for name, op in ops:
            vv, cv, cc = self.operator(op)
            out[name] = self.ortho_pack(False, vv, cv, cc, cvS)
        terms = range(self.pot_dim) if terms is None else terms
        for j in terms:
            vv, cv, cc = self.operator(OP_ELECPOT, j)
            out[f"V{j}"] = self.ortho_pack(False, vv, cv, cc, cvS)
        return out


def state_offsets(system):
    """First valence and core state of every atom: the valence-first
    numbering of cumulValeStates / cumulCoreStates (atomicSites.f90:132-137)."""
    nv = np.array([system.types[t].num_vale_states for t in system.site_type])
    nc = np.array([system.types[t].num_core_states for t in system.site_type])
    cv = np.concatenate([[0], np.cumsum(nv)])
    cc = np.concatenate([[0], np.cumsum(nc)])
    return cv, cc


def ortho_pack_blas(is_overlap: bool, vv, cv, cc, scv) -> np.ndarray:
    """orthoOL / ortho(opCode) of integrals.F90:2601-2853 with intgOrtho.F90:23-187
    restated with matrix products (the reference itself calls zherk/zher2k
    for the first term):

        O' = O_vv - (S_cv^H O_cv + O_cv^H S_cv) + S_cv^H O_cc S_cv
        S' = S_vv - 2 S_cv^H S_cv               + S_cv^H S_cc S_cv

    upper triangle, the diagonal of the first update made real (zherk /
    zher2k), packed column by column, |re|, |im| < 1e-10 flushed to zero when
    there are core states (intgOrtho.F90:178-183).  Array shapes as
    Oracle.operator returns them ([nk, cols, rows] memory order); the same
    numbers as Oracle.ortho_pack up to the order of the sums, fast enough for
    the largest workloads."""
    nk, nv = vv.shape[0], vv.shape[1]
    rows, cols = packed_index(nv)
    out = np.zeros((nk, nv * (nv + 1) // 2, 2))
    for q in range(nk):
        V = vv[q].T
        if cv is None or cv.shape[2] == 0:
            vals = V[rows, cols]
            out[q, :, 0], out[q, :, 1] = vals.real, vals.imag
            continue
        Sm = scv[q].T                       # [nc, nv]
        Om = cv[q].T
        if is_overlap:
            T1 = -2.0 * (Sm.conj().T @ Sm)
        else:
            T1 = -(Sm.conj().T @ Om + Om.conj().T @ Sm)
        W = V + T1
        d = np.arange(nv)
        W[d, d] = V[d, d].real + T1[d, d].real
        W = W + (Sm.conj().T @ cc[q].T) @ Sm
        vals = W[rows, cols]
        re, im = vals.real.copy(), vals.imag.copy()
        re[np.abs(re) < 1.0e-10] = 0.0
        im[np.abs(im) < 1.0e-10] = 0.0
        out[q, :, 0], out[q, :, 1] = re, im
    return out


def assemble(packed: Dict[str, np.ndarray], coeffs: np.ndarray) -> np.ndarray:
    """secularEqn.F90:128-150 with readPackedMatrixAccum's rule that a zero
    multiplier adds the term unscaled (matrixSubs.F90:278-282); the mass
    velocity joins when present (rel = 1, :137-143)."""
    h = packed["NP"].copy()
    h = h + packed["KE"]
    if "MV" in packed:
        h = h + packed["MV"]
    for j, c in enumerate(coeffs):
        v = packed[f"V{j}"]
        h = h + v if c == 0.0 else h + v * c
    return h


def unpack(packed_k: np.ndarray, n: int) -> np.ndarray:
    """unpackMatrix with fullFlag=1 (matrixSubs.F90:314-341): Hermitian full."""
    m = np.zeros((n, n), np.complex128)
    iu = np.triu_indices(n)
    # packed order: column i, rows j <= i  -> (j, i)
    cols = np.concatenate([np.full(i + 1, i) for i in range(n)])
    rows = np.concatenate([np.arange(i + 1) for i in range(n)])
    vals = packed_k[:, 0] + 1j * packed_k[:, 1]
    m[rows, cols] = vals
    m[cols, rows] = np.conj(vals)
    m[np.arange(n), np.arange(n)] = packed_k[[(i * (i + 3)) // 2 for i in range(n)], 0]
    del iu
    return m


def zhegv(h_packed: np.ndarray, s_packed: np.ndarray, n: int, num_states: int):
    """Eigenvalues/vectors per k with LAPACK zhegv (itype 1, 'V', 'U')."""
    import scipy.linalg as sl
    nk = h_packed.shape[0]
    w = np.zeros((nk, num_states))
    vecs = np.zeros((nk, n, num_states), np.complex128)
    for q in range(nk):
        H = unpack(h_packed[q], n)
        S = unpack(s_packed[q], n)
        ev, Z = sl.eigh(H, S, type=1, driver="gv", lower=False)
        w[q] = ev[:num_states]
        vecs[q] = Z[:, :num_states]
    return w, vecs


# ---- valence charge (the step after the eigen-solve) ------------------------
SMALL_THRESH = 1.0e-8          # smallThresh, src/constants.f90:49


def packed_index(n: int):
    """(rows, cols) of the upper-packed order: column i, rows j <= i."""
    cols = np.concatenate([np.full(i + 1, i) for i in range(n)])
    rows = np.concatenate([np.arange(i + 1) for i in range(n)])
    return rows, cols


def matrix_element_mult(m1: np.ndarray, m2: np.ndarray) -> float:
    """matrixElementMult (src/olcao/matrixSubs.F90:10-53) on packed [plen, 2]
    arrays: off-diagonal elements contribute re*re + im*im, the diagonal only
    re*re / 2, and the sum is doubled for the lower half."""
    plen = m1.shape[0]
    n = int(round((np.sqrt(8 * plen + 1) - 1) / 2))
    diag = np.array([i * (i + 3) // 2 for i in range(n)])
    prod = m1[:, 0] * m2[:, 0] + m1[:, 1] * m2[:, 1]
    off = prod.sum() - prod[diag].sum()
    return 2.0 * (off + (m1[diag, 0] * m2[diag, 0]).sum() / 2.0)


def make_valence_rho(packed: Dict[str, np.ndarray], pot_dim: int, occupation: np.ndarray,
                     eigenvalues: np.ndarray, vectors: np.ndarray):
    """makeValenceRho (src/olcao/valeCharge.F90:172-395) for stored operators.

    occupation, eigenvalues: [spin, nk, num_states] (the reference's
    (numStates, numKPoints, spin) in memory order); vectors [spin, nk,
    num_states, n] complex (valeVale(:, state) per k).  Per k: the states
    with sum_s |f| >= smallThresh (:234) add f * lambda to the electron
    energy and f x x^H to rho's upper triangle (zher, :240); rho is packed,
    for spin 2 turned into (up + down, up - down) (:307-313), and traced with
    S, NP, KE and every V_j (:321-395).

    Returns (traces [spin, 3 + rel + pot_dim] = charge, nuclear, kinetic,
    mass velocity (when packed holds "MV"), potRho; electron energy [spin];
    packed rho [spin, nk, plen, 2])."""
    spin, nk, ns = occupation.shape
    n = vectors.shape[-1]
    rows, cols = packed_index(n)
    names = ["S", "NP", "KE"] + (["MV"] if "MV" in packed else []) + [f"V{j}" for j in range(pot_dim)]
    traces = np.zeros((spin, len(names)))
    energy = np.zeros(spin)
    rho_packed = np.zeros((spin, nk, rows.size, 2))
    for k in range(nk):
        keep = [j for j in range(ns) if np.abs(occupation[:, k, j]).sum() >= SMALL_THRESH]
        for j in keep:
            energy += occupation[:, k, j] * eigenvalues[:, k, j]
        pk = []
        for s in range(spin):
            X = vectors[s, k][keep].T                      # [n, nocc]
            R = (X * occupation[s, k, keep][None, :]) @ X.conj().T
            v = R[rows, cols]
            pk.append(np.stack([v.real, v.imag], -1))
        if spin == 2:
            pk = [pk[0] + pk[1], pk[0] - pk[1]]
        for s in range(spin):
            rho_packed[s, k] = pk[s]
            for t, name in enumerate(names):
                traces[s, t] += matrix_element_mult(packed[name][k], pk[s])
    return traces, energy, rho_packed


def massvel_scale(a1: float, a2: float, A, B, l1: int, l2: int) -> float:
    """Rounding scale of a mass-velocity block: the largest Cartesian element
    of (alpha^2/8) <a|nabla^4|b> with every term of its expansion in 1-D
    overlaps (the one prim_massvel evaluates) taken in absolute value.  Two
    correct FP64 evaluations of the block agree to a small multiple of
    2^-52 times this; with very unequal exponents the terms cancel to many
    digits, so the block itself can be far smaller than the scale."""
    A = np.asarray(A, float)
    B = np.asarray(B, float)
    z = a1 + a2
    inv2z = 1.0 / (2.0 * z)
    xi = a1 * a2 / z
    P = (a1 * A + a2 * B) / z
    pref = (np.pi / z) ** 1.5 * np.exp(-xi * np.sum((A - B) ** 2))
    tabs = []
    for c in range(3):
        pa, pb = abs(P[c] - A[c]), abs(P[c] - B[c])
        s = np.zeros((l1 + 1, l2 + 5))
        s[0, 0] = 1.0
        for i in range(l1 + 1):
            if i > 0:
                s[i, 0] = pa * s[i - 1, 0] + ((i - 1) * inv2z * s[i - 2, 0] if i > 1 else 0.0)
            for j in range(1, l2 + 5):
                v = pb * s[i, j - 1]
                if i > 0:
                    v += i * inv2z * s[i - 1, j - 1]
                if j > 1:
                    v += (j - 1) * inv2z * s[i, j - 2]
                s[i, j] = v
        tabs.append(s)

    def d2(j):
        out = [(j, 2 * a2 * (2 * j + 1)), (j + 2, 4 * a2 * a2)]
        return out + ([(j - 2, j * (j - 1))] if j >= 2 else [])

    def lap(s, i, j):
        return sum(w * s[i, m] for m, w in d2(j))

    def lap2(s, i, j):
        return sum(w * lap(s, i, m) for m, w in d2(j))

    def cart(l):
        return [(x, y, n - x - y) for n in range(l + 1) for x in range(n, -1, -1) for y in range(n - x, -1, -1)]

    best = 0.0
    for ea in cart(l1):
        for eb in cart(l2):
            i0 = [tabs[c][ea[c], eb[c]] for c in range(3)]
            i2 = [lap(tabs[c], ea[c], eb[c]) for c in range(3)]
            i4 = [lap2(tabs[c], ea[c], eb[c]) for c in range(3)]
            v = (i4[0] * i0[1] * i0[2] + i0[0] * i4[1] * i0[2] + i0[0] * i0[1] * i4[2]
                 + 2 * (i2[0] * i2[1] * i0[2] + i2[0] * i0[1] * i2[2] + i0[0] * i2[1] * i2[2]))
            best = max(best, v)
    return 3.0 * best * pref * (7.2973525693e-3) ** 2 / 8.0


# ---- occupations (the step before the valence density) ----------------------
def merge_sort(values):
    """The reference's bottom-up merge of adjacent runs (sortSubs.f90:18-175),
    ties taken from the second run first.  Returns (sorted, order)."""
    n = len(values)
    a, oa = list(values), list(range(n))
    b, ob = [0.0] * n, [0] * n
    borders = list(range(n + 1))
    nseg = n
    src_a = True
    while nseg > 1:
        fd, fo, td, to = (a, oa, b, ob) if src_a else (b, ob, a, oa)
        tp = 0
        for i in range(nseg // 2):
            p1, p2 = borders[2 * i], borders[2 * i + 1]
            e1, e2 = borders[2 * i + 1], borders[2 * i + 2]
            while tp < e2:
                if p1 < e1 and (p2 >= e2 or fd[p1] < fd[p2]):
                    td[tp], to[tp] = fd[p1], fo[p1]
                    p1 += 1
                else:
                    td[tp], to[tp] = fd[p2], fo[p2]
                    p2 += 1
                tp += 1
            borders[i + 1] = e2
        if nseg % 2:
            for q in range(tp, borders[nseg]):
                td[q], to[q] = fd[q], fo[q]
            borders[nseg // 2 + 1] = borders[nseg]
        src_a = not src_a
        nseg = nseg // 2 + nseg % 2
    return (a, oa) if src_a else (b, ob)


def populate_states(eigenvalues: np.ndarray, kpoint_weights: np.ndarray, num_electrons: float,
                    thermal_sigma: float = 0.0, fermi_search_limit: float = 0.5,
                    max_thermal_range: float = 11.5):
    """populateStates (src/olcao/populate.F90:132-578): populateStandard,
    then populateSmearing when thermal_sigma != 0.  eigenvalues [spin, nk,
    num_states]; returns (occupation of that shape, occupied energy)."""
    spin, nk, ns = eigenvalues.shape
    vals, kpt = [], []
    for k in range(nk):                   # k-point, spin, state (:224-232)
        for s in range(spin):
            for j in range(ns):
                vals.append(float(eigenvalues[s, k, j]))
                kpt.append(k)
    srt, order = merge_sort(vals)
    n = len(vals)

    def w(i):
        return kpoint_weights[kpt[order[i]]] / spin

    pop = [0.0] * n
    placed = 0.0
    occ = None
    for i in range(n):                    # :292-331
        pop[order[i]] = w(i)
        placed += pop[order[i]]
        if placed > num_electrons:
            pop[order[i]] = w(i) + num_electrons - placed
            placed = num_electrons
        if abs(num_electrons - placed) < SMALL_THRESH:
            occ = i
            break
    if occ is None:
        raise ValueError("the states hold fewer electrons than num_electrons")
    e_occ = srt[occ]
    lo = hi = occ                          # degenerate top level (:344-399)
    charge, possible = pop[order[occ]], w(occ)
    while hi + 1 < n and abs(e_occ - srt[hi + 1]) <= SMALL_THRESH:
        hi += 1
        possible += w(hi)
    while lo > 0 and abs(e_occ - srt[lo - 1]) <= SMALL_THRESH:
        lo -= 1
        possible += w(lo)
        charge += w(lo)
    for i in range(lo, hi + 1):
        pop[order[i]] = charge / possible * w(i)
    occ = hi
    e_occ = srt[occ]
    if thermal_sigma != 0.0:               # :484-576
        emin = srt[occ] - fermi_search_limit
        emax = srt[min(occ + 1, n - 1)] + fermi_search_limit
        for _ in range(500):
            e_occ = 0.5 * (emin + emax)
            total = 0.0
            pop = [0.0] * n
            for i in range(n):
                x = (srt[i] - e_occ) / thermal_sigma
                f = 0.0 if x > max_thermal_range else 1.0 if x < -max_thermal_range else 1.0 / (1.0 + math.exp(x))
                if f == 0.0:
                    break
                pop[order[i]] = w(i) * f
                total += pop[order[i]]
            if abs(total - num_electrons) < SMALL_THRESH:
                break
            if total < num_electrons:
                emin = e_occ
            else:
                emax = e_occ
    out = np.zeros_like(eigenvalues, dtype=np.float64)
    q = 0
    for k in range(nk):
        for s in range(spin):
            for j in range(ns):
                out[s, k, j] = pop[q]
                q += 1
    return out, e_occ
