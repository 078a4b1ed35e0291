"""Python front end of libolcao_gb300 (C ABI in include/olcao_gpu.h).

Mirrors the reference's module procedures for the hot path:

=========================  ==================================================
this module                reference (src/olcao/...)
=========================  ==================================================
``Context(system)``        setupSCF set-up: initializeLattice, computePhase-
                           Factors, renormalizeBasis, makeAlpha*Dist
``gauss_overlap(OL)``      gaussOverlapOL     integrals.F90:81-486
``gauss_overlap(KE)``      gaussOverlapKE     integrals.F90:490-900
``gauss_overlap(MV)``      gaussOverlapMV     integrals.F90:904-1320
``gauss_overlap(NP)``      gaussOverlapNP     integrals.F90:1324-1715
``gauss_overlap(EP, j)``   gaussOverlapEP     integrals.F90:1719-2122
``ortho_pack``             orthoOL / ortho    integrals.F90:2601-2853
``assemble_hamiltonian``   secularEqn H build secularEqn.F90:128-166
``solve_zhegv``            solveZHEGV         interfaces.F90:73-120
``scf_iteration``          secularEqnAllKP with the potential-dependent
                           integrals recomputed (fused form)
``populate_states``        populateStates     populate.F90:132-578
``make_valence_rho``       makeValenceRho     valeCharge.F90:34-420
=========================  ==================================================

Device buffers are torch CUDA tensors (torch is only the allocator and
stream provider).  There is no CPU fallback: when the compiled library is
missing every call raises.
"""

from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libolcao_gb300.so")

OP_OVERLAP, OP_KINETIC, OP_NUCLEAR, OP_ELECPOT, OP_MASSVEL, OP_HAMILTONIAN = 1, 2, 3, 4, 5, 6
PREC_FP64, PREC_MIXED = 0, 1
FORM_FUSED, FORM_STORED = 0, 1
ITER_EIG_DEVICE, ITER_COEFF_DEVICE, ITER_GRAPH = 1, 2, 4

EXPORTS = ("olc_version", "olc_last_error", "olc_create", "olc_destroy",
           "olc_get_dims", "olc_set_stream", "olc_gauss_overlap",
           "olc_ortho_pack", "olc_assemble_hamiltonian", "olc_solve_zhegv",
           "olc_scf_prepare", "olc_scf_iteration", "olc_primitive_batch",
           "olc_profile_enable", "olc_profile_reset", "olc_profile_read",
           "olc_launch_count", "olc_profile_read_work", "olc_scf_matrices", "olc_solve_zhegv_noalloc",
           "olc_split_zgemm", "olc_split_cgemm32", "olc_write_setup_integrals", "olc_write_eigen",
           "olc_make_valence_rho", "olc_populate_states")
STAGES = ("primitives", "contract", "bloch", "ortho", "assemble", "solve", "refine",
          "density", "tridiag", "backtransform", "split")

_LIB: Optional[C.CDLL] = None


class OlcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"olcao_gb300 status {status}: {msg}")
        self.status = status


class Dims(C.Structure):
    _fields_ = [("vale_dim", C.c_int32), ("core_dim", C.c_int32),
                ("pot_dim", C.c_int32), ("num_kpoints", C.c_int32),
                ("num_cells", C.c_int32), ("num_pair_tasks", C.c_int32),
                ("packed_len", C.c_int64)]


def lib() -> C.CDLL:
    """Load the compiled library; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise OlcError(-1, f"{LIB_PATH} is missing: run olcao_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        vp, i32, dp = C.c_void_p, C.c_int, C.c_void_p
        L.olc_version.restype = C.c_char_p
        L.olc_last_error.argtypes = [C.c_char_p, C.c_size_t]
        L.olc_create.argtypes = [vp, vp, C.POINTER(vp)]
        L.olc_destroy.argtypes = [vp]
        L.olc_get_dims.argtypes = [vp, C.POINTER(Dims)]
        L.olc_set_stream.argtypes = [vp, vp]
        L.olc_gauss_overlap.argtypes = [vp, i32, i32, dp, i32, dp, dp, dp]
        L.olc_ortho_pack.argtypes = [vp, i32, dp, dp, dp, dp, dp]
        L.olc_assemble_hamiltonian.argtypes = [vp, dp, dp, i32, dp]
        L.olc_solve_zhegv.argtypes = [vp, dp, dp, i32, dp, dp, dp]
        L.olc_scf_prepare.argtypes = [vp, i32, i32]
        L.olc_scf_iteration.argtypes = [vp, dp, i32, i32, dp, i32, dp]
        L.olc_primitive_batch.argtypes = [i32, i32, dp, dp, dp]
        L.olc_profile_enable.argtypes = [vp, i32]
        L.olc_profile_reset.argtypes = [vp]
        L.olc_profile_read.argtypes = [vp, i32, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.olc_profile_read_work.argtypes = [vp, i32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        for name in EXPORTS[2:]:
            getattr(L, name).restype = C.c_int
        L.olc_scf_matrices.argtypes = [vp, dp, i32, dp, dp, i32]
        L.olc_solve_zhegv_noalloc.argtypes = [i32, i32, dp, dp, i32, dp, dp, dp, vp]
        L.olc_split_zgemm.argtypes = [vp, i32, i32, i32, dp, dp, dp]
        L.olc_split_cgemm32.argtypes = [vp, i32, i32, i32, dp, i32, dp, dp]
        L.olc_write_setup_integrals.argtypes = [vp, C.c_char_p]
        L.olc_write_eigen.argtypes = [C.c_char_p, i32, i32, i32, i32, dp, dp]
        L.olc_make_valence_rho.argtypes = [vp, i32, i32, dp, dp, dp, dp, dp, dp]
        d = C.c_double
        L.olc_populate_states.argtypes = [i32, i32, i32, dp, dp, d, d, d, d, dp, dp]
        L.olc_launch_count.restype = C.c_int64
        L.olc_launch_count.argtypes = []
        _LIB = L
    return _LIB


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().olc_last_error(buf, 1024)
    return buf.value.decode()


def _check(status: int):
    if status != 0:
        raise OlcError(status, last_error())


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def launch_count() -> int:
    """Kernels of this library launched so far in the process."""
    return int(lib().olc_launch_count())


def primitive_batch(kind: int, params: np.ndarray, lmalpha: np.ndarray) -> np.ndarray:
    """Evaluate primitive sh(16,16) blocks on the device (kind 1 overlap,
    2 kinetic, 3 nuclear, 4 electron 3-centre, 5 mass velocity, 6 / 7 / 8
    the x / y / z momentum component); returns [n, 16, 16] indexed
    [item, row lm1, col lm2]."""
    p = np.ascontiguousarray(params, np.float64)
    lm = np.ascontiguousarray(lmalpha, np.int32)
    n = p.shape[0]
    out = np.zeros((n, 256))
    _check(lib().olc_primitive_batch(kind, n, p.ctypes.data, lm.ctypes.data, out.ctypes.data))
    return out.reshape(n, 16, 16).transpose(0, 2, 1)


def write_eigen(root: str, eigenvalues: np.ndarray, vectors: Optional[np.ndarray] = None,
                spin: int = 1) -> None:
    """Write eigenvalues [nk, num_states] and (optionally) eigenvectors
    [nk, num_states, vale_dim] complex in the reference's main-temp.hdf5
    dataset layout (raw files + manifest.json under root)."""
    ev = np.ascontiguousarray(eigenvalues, np.float64)
    nk, ns = ev.shape
    vp = None
    nv = ns
    if vectors is not None:
        vc = np.ascontiguousarray(vectors, np.complex128)
        assert vc.shape[:2] == (nk, ns)
        nv = vc.shape[2]
        vp = vc.ctypes.data
    _check(lib().olc_write_eigen(root.encode(), nk, spin, ns, nv, ev.ctypes.data, vp))


def populate_states(eigenvalues, kpoint_weights, num_electrons: float,
                    thermal_sigma: float = 0.0, fermi_search_limit: float = 0.5,
                    max_thermal_range: float = 11.5):
    """populateStates (populate.F90:132-578) on host arrays: eigenvalues
    [spin, nk, num_states] or [nk, num_states] (Hartree), kpoint_weights [nk].
    Returns (occupation of the same shape as eigenvalues, occupied energy)."""
    ev = np.ascontiguousarray(eigenvalues, np.float64)
    squeeze = ev.ndim == 2
    if squeeze:
        ev = ev[None]
    spin, nk, ns = ev.shape
    kw = np.ascontiguousarray(kpoint_weights, np.float64)
    if kw.shape != (nk,):
        raise ValueError(f"kpoint_weights has shape {kw.shape}, expected ({nk},)")
    occ = np.zeros_like(ev)
    ef = C.c_double()
    _check(lib().olc_populate_states(ns, nk, spin, ev.ctypes.data, kw.ctypes.data, float(num_electrons),
                                     float(thermal_sigma), float(fermi_search_limit),
                                     float(max_thermal_range), occ.ctypes.data, C.addressof(ef)))
    return (occ[0] if squeeze else occ), float(ef.value)


def read_dataset(root: str, path: str) -> np.ndarray:
    """One dataset written by the raw writers, as an array of its HDF5 dims
    (Fortran order), found through root/manifest.json."""
    import json
    import os
    with open(os.path.join(root, "manifest.json")) as f:
        man = json.load(f)
    for d in man["datasets"]:
        if d["path"] == path:
            data = np.fromfile(os.path.join(root, d["file"]), dtype="<f8")
            return data.reshape(d["dims"], order="F")
    raise KeyError(path)


class Context:
    """One system on the current CUDA device (olc_create)."""

    def __init__(self, system, stream=None):
        import torch
        self.torch = torch
        self.system = system
        self._struct = system.to_struct()
        h = C.c_void_p()
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _check(lib().olc_create(C.byref(self._struct), C.c_void_p(s), C.byref(h)))
        self.h = h
        d = Dims()
        _check(lib().olc_get_dims(h, C.byref(d)))
        self.rel = int(getattr(system, "rel", 0))
        self.vale_dim, self.core_dim = d.vale_dim, d.core_dim
        self.pot_dim, self.nk = d.pot_dim, d.num_kpoints
        self.num_cells, self.num_pair_tasks = d.num_cells, d.num_pair_tasks
        self.packed_len = d.packed_len

    def close(self):
        if getattr(self, "h", None):
            lib().olc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def profile(self, on: bool = True):
        _check(lib().olc_profile_enable(self.h, int(on)))

    def profile_reset(self):
        _check(lib().olc_profile_reset(self.h))

    def profile_read(self) -> Dict[str, Tuple[int, float]]:
        """{stage: (kernel launches, milliseconds)} since the last reset."""
        out = {}
        for i, name in enumerate(STAGES):
            n = C.c_int64()
            ms = C.c_double()
            _check(lib().olc_profile_read(self.h, i, C.byref(n), C.byref(ms)))
            out[name] = (int(n.value), float(ms.value))
        return out

    def profile_work(self) -> Dict[str, Tuple[float, float]]:
        """{stage: (tensor flops, streamed bytes)} since the last reset."""
        out = {}
        for i, name in enumerate(STAGES):
            fl = C.c_double()
            by = C.c_double()
            _check(lib().olc_profile_read_work(self.h, i, C.byref(fl), C.byref(by)))
            out[name] = (float(fl.value), float(by.value))
        return out

    def set_stream(self, stream):
        _check(lib().olc_set_stream(self.h, C.c_void_p(stream.cuda_stream)))

    # -- buffers ---------------------------------------------------------------
    def _z(self, *shape):
        return self.torch.zeros(*shape, dtype=self.torch.complex128, device="cuda")

    def blocks(self):
        nv, nc, nk = self.vale_dim, self.core_dim, self.nk
        vv = self._z(nk, nv, nv)
        cv = self._z(nk, nv, nc) if nc else None
        cc = self._z(nk, nc, nc) if nc else None
        return vv, cv, cc

    # -- reference module procedures ------------------------------------------
    def gauss_overlap(self, op: int, term: int = 0, coeffs=None,
                      precision: int = PREC_FP64, out=None):
        """One integral pass; returns (vv, cv, cc) device tensors shaped
        [nk, cols, rows] (the reference's column-major (rows, cols, nk))."""
        vv, cv, cc = out if out is not None else self.blocks()
        cptr = None
        if coeffs is not None:
            carr = np.ascontiguousarray(coeffs, np.float64)
            cptr = carr.ctypes.data
        _check(lib().olc_gauss_overlap(self.h, op, term, cptr, precision, _ptr(vv),
                                       _ptr(cv), _ptr(cc)))
        return vv, cv, cc

    def ortho_pack(self, is_overlap: bool, vv, cv, cc, scv):
        packed = self.torch.zeros(self.nk, self.packed_len, 2, dtype=self.torch.float64,
                                  device="cuda")
        _check(lib().olc_ortho_pack(self.h, int(is_overlap), _ptr(vv), _ptr(cv), _ptr(cc),
                                    _ptr(scv), _ptr(packed)))
        return packed

    def packed_operators(self, terms: Optional[Sequence[int]] = None) -> Dict[str, object]:
        """OLCAOsetup's stored integrals: packed, orthogonalised S, KE, NP, V_j."""
        vvS, cvS, ccS = self.gauss_overlap(OP_OVERLAP)
        out = {"S": self.ortho_pack(True, vvS.clone(), cvS, ccS, cvS)}
        ops = (("KE", OP_KINETIC), ("NP", OP_NUCLEAR)) + ((("MV", OP_MASSVEL),) if self.rel else ())
        for name, op in ops:
            vv, cv, cc = self.gauss_overlap(op)
            out[name] = self.ortho_pack(False, vv, cv, cc, cvS)
        terms = range(self.pot_dim) if terms is None else terms
        for j in terms:
            vv, cv, cc = self.gauss_overlap(OP_ELECPOT, j)
            out[f"V{j}"] = self.ortho_pack(False, vv, cv, cc, cvS)
        return out

    def assemble_hamiltonian(self, packed: Dict[str, object], coeffs) -> object:
        fixed = [packed["NP"], packed["KE"]] + ([packed["MV"]] if "MV" in packed else [])
        terms = fixed + [packed[f"V{j}"] for j in range(self.pot_dim)]
        co = np.concatenate([np.ones(len(fixed)), np.asarray(coeffs, np.float64)])
        ptrs = (C.c_void_p * len(terms))(*[t.data_ptr() for t in terms])
        out = self.torch.empty_like(packed["NP"])
        _check(lib().olc_assemble_hamiltonian(self.h, C.cast(ptrs, C.c_void_p),
                                              co.ctypes.data, len(terms), out.data_ptr()))
        return out

    def solve_zhegv(self, packed_h, packed_s, num_states: int, vectors: bool = False):
        torch = self.torch
        eig = torch.zeros(self.nk, num_states, dtype=torch.float64, device="cuda")
        vec = (torch.zeros(self.nk, num_states, self.vale_dim, dtype=torch.complex128,
                           device="cuda") if vectors else None)
        info = np.zeros(self.nk, np.int32)
        _check(lib().olc_solve_zhegv(self.h, packed_h.data_ptr(), packed_s.data_ptr(),
                                     num_states, eig.data_ptr(), _ptr(vec), info.ctypes.data))
        return eig, vec, info

    def scf_prepare(self, precision: int = PREC_FP64, form: int = FORM_FUSED):
        _check(lib().olc_scf_prepare(self.h, precision, form))

    def write_setup_integrals(self, root: str):
        """Packed orthogonalised S, KE, NP and V_j of every k in the
        reference's setup-temp.hdf5 dataset layout (after
        scf_prepare(..., FORM_STORED))."""
        _check(lib().olc_write_setup_integrals(self.h, root.encode()))

    def split_zgemm(self, A, B):
        """FP64-accurate complex product on the tensor cores (device tensors,
        row-major numpy-style [rows, cols]; computed column-major inside)."""
        torch = self.torch
        m, k = A.shape
        k2, n = B.shape
        assert k == k2
        Ac = A.t().contiguous()        # column-major storage of A
        Bc = B.t().contiguous()
        Cc = torch.zeros(n, m, dtype=torch.complex128, device="cuda")
        _check(lib().olc_split_zgemm(self.h, m, n, k, Ac.data_ptr(), Bc.data_ptr(),
                                     Cc.data_ptr()))
        return Cc.t()

    def split_cgemm32(self, A, B, conj_a: bool = False):
        """FP32-accurate complex product op(A) B on the tensor cores (device
        complex64 tensors, row-major numpy-style; op(A) = A or A^H)."""
        torch = self.torch
        if conj_a:
            k, m = A.shape
        else:
            m, k = A.shape
        k2, n = B.shape
        assert k == k2
        Ac = A.t().contiguous()        # column-major storage of A
        Bc = B.t().contiguous()
        Cc = torch.zeros(n, m, dtype=torch.complex64, device="cuda")
        _check(lib().olc_split_cgemm32(self.h, m, n, k, Ac.data_ptr(), int(conj_a), Bc.data_ptr(),
                                       Cc.data_ptr()))
        return Cc.t()

    def scf_matrices(self, coeffs, k: int):
        """Full Hermitian H(k), S(k) of the prepared pass, as host arrays."""
        co = np.ascontiguousarray(coeffs, np.float64)
        n = self.vale_dim
        H = np.zeros((n, n), np.complex128)
        Sm = np.zeros((n, n), np.complex128)
        _check(lib().olc_scf_matrices(self.h, co.ctypes.data, k, H.ctypes.data,
                                      Sm.ctypes.data, 0))
        # memory is column-major: transpose to [row, col]
        return H.T.copy(), Sm.T.copy()

    def scf_iteration(self, coeffs, num_states: int, precision: int = PREC_FP64,
                      eig_out=None, vectors=None, graph: bool = False):
        """One SCF pass; returns eigenvalues [nk, num_states].  coeffs and
        eig_out may each be host numpy arrays or device tensors.  graph=True
        runs the mixed stored-form pass as a CUDA graph (captured on the
        second call for a given num_states / vectors choice)."""
        flags = ITER_GRAPH if graph else 0
        if isinstance(coeffs, np.ndarray) or not hasattr(coeffs, "data_ptr"):
            co = np.ascontiguousarray(coeffs, np.float64)
            cptr = co.ctypes.data
        else:
            co = coeffs
            cptr = coeffs.data_ptr()
            flags |= ITER_COEFF_DEVICE
        if eig_out is None:
            eig_out = np.zeros((self.nk, num_states))
        if not isinstance(eig_out, np.ndarray):
            flags |= ITER_EIG_DEVICE
        _check(lib().olc_scf_iteration(self.h, cptr, precision, num_states,
                                       _ptr(eig_out), flags, _ptr(vectors)))
        return eig_out

    def make_valence_rho(self, occupation, vectors, eigenvalues=None, rho: bool = False):
        """makeValenceRho (valeCharge.F90:34-420) on the prepared operators.

        occupation (and eigenvalues, optional) are host arrays [spin, nk,
        num_states] or [nk, num_states] for spin 1: the reference's
        structuredElectronPopulation, occupation times k-point weight.
        vectors is a device complex128 tensor [spin, nk, num_states, n] (or
        [nk, num_states, n]) as scf_iteration fills it.  Returns (traces
        [spin, 3 + rel + pot_dim] = chargeDensityTrace, nucPotTrace,
        kineticEnergyTrace, massVelocityTrace (rel = 1 only), potRho(1..pot_dim)
        per spin column (total, difference); electronEnergy [spin] or None;
        packed rho tensor [spin, nk, packed_len, 2] or None)."""
        torch = self.torch
        occ = np.ascontiguousarray(occupation, np.float64)
        if occ.ndim == 2:
            occ = occ[None]
        spin, nk, ns = occ.shape
        if nk != self.nk:
            raise ValueError(f"occupation has {nk} k-points, the context {self.nk}")
        if tuple(vectors.shape[-3:]) != (nk, ns, self.vale_dim) or vectors.numel() != spin * nk * ns * self.vale_dim:
            raise ValueError(f"vectors shape {tuple(vectors.shape)} does not match occupation {occ.shape}")
        if vectors.dtype != torch.complex128 or not vectors.is_contiguous():
            raise ValueError("vectors must be a contiguous complex128 device tensor")
        eig = None
        if eigenvalues is not None:
            eig = np.ascontiguousarray(eigenvalues, np.float64).reshape(occ.shape)
        traces = np.zeros((spin, 3 + self.rel + self.pot_dim))
        energy = np.zeros(spin) if eig is not None else None
        rp = (torch.zeros(spin, nk, self.packed_len, 2, dtype=torch.float64, device="cuda")
              if rho else None)
        _check(lib().olc_make_valence_rho(self.h, ns, spin, occ.ctypes.data, _ptr(eig),
                                          vectors.data_ptr(), traces.ctypes.data, _ptr(energy),
                                          _ptr(rp)))
        return traces, energy, rp
