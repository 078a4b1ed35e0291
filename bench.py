#!/usr/bin/env python
"""Seconds per SCF iteration of OLCAO's hot path on one GB300.

Workload (default): the Si64 configuration -- a 2x2x2 conventional diamond Si
supercell (64 atoms, a = 5.431 A, seeded displacements sigma = 0.03 A), 1s2s2p
core + 3s3p3d4s4p valence per atom (832 valence / 320 core basis functions),
18 even-tempered Gaussians 0.12..1e6, a 16-term site potential, 4x4x4
Monkhorst-Pack mesh (64 k-points), complex128 H(k), S(k).

One step is one SCF iteration of the reference's secularEqnAllKP: H(k) =
NP + KE + sum_j c_j V_j assembled from the orthogonalised, packed integrals
(computed once by the integral kernels and kept resident in HBM, as
OLCAOsetup stores them), then the generalised eigen-problem with eigenvectors
for every k.  The potential coefficients change every step.  The resident
integrals (~6.7 GB) exceed L2, so no flush is needed between steps.

The headline is the mixed+batched form (FP32 solves, Rayleigh-Ritz with
error-free split-BF16 tensor-core products); the same run times the plain
FP64 GPU path and reports the largest eigenvalue difference between them.

--impl reference times the CPU restatement of the same iteration (assembly +
LAPACK zhegv per k) on the host cores, on a bounded sample of k-points.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "s per SCF iteration, mixed+batched vs FP64 GPU path at ≤1e-6 Ha eigenvalue error"
WORKLOADS = {
    "si64": "Si64 2x2x2 diamond supercell, 832 basis fns (320 core), 64 k (4x4x4 MP), "
            "18 Gaussians 0.12-1e6, 16-term potential",
    "diamond": "diamond C 2-atom FCC, 10 basis fns (2 core), 216 k (6x6x6 MP)",
    "si8": "Si8 conventional cell, valence only, 104 basis fns, 512 k (8x8x8 MP)",
    "graphite": "AB graphite 4 atoms, valence only, 32 basis fns, 8192 k (32x32x8 MP)",
    "quartz": "alpha-quartz SiO2 3x3x3 (243 atoms), 3159 basis fns (567 core), 9 k (Gamma + 2x2x2)",
    "si512": "Si512 4x4x4 diamond supercell, 6656 basis fns (2560 core), 9 k (Gamma + shifted 2x2x2)",
    "batched": "uneven batch: AB graphite (n = 32, 8192 k) and Si8 (n = 104, 512 k), "
               "one mixed pass of each per step (two passes back to back, not one launch)",
}
BATCHED_PARTS = ("graphite", "si8")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="si512", choices=sorted(WORKLOADS))
    p.add_argument("--form", default="stored", choices=["stored", "fused"])
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--no-fused", action="store_true", help="skip the fused-form timing")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-fp64", action="store_true",
                   help="profiling runs only: skip the plain FP64 GPU comparison")
    p.add_argument("--no-graph", action="store_true",
                   help="launch the mixed pass directly instead of replaying its CUDA graph")
    p.add_argument("--cpu-sample-k", type=int, default=2)
    p.add_argument("--nk", type=int, default=0,
                   help="profiling runs only: keep the first NK k-points")
    p.add_argument("--k-stride", type=int, default=1,
                   help="with --valence-rho-only: keep every K_STRIDE-th k-point")
    p.add_argument("--valence-rho-only", action="store_true",
                   help="profiling runs only: prepare, one pass with vectors, then two "
                        "olc_make_valence_rho calls between cudaProfilerStart/Stop")
    return p.parse_args()


def run_valence_rho_only(args):
    """The density step alone, for ncu (--profile-from-start off) captures."""
    import torch
    from olcao_gb300 import api
    from olcao_gb300 import system as S
    sysm = S.SYSTEMS[args.config]()
    sysm.kpoints_abc = sysm.kpoints_abc[::args.k_stride]
    if args.nk > 0:
        sysm.kpoints_abc = sysm.kpoints_abc[:args.nk]
    ctx = api.Context(sysm)
    ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
    n, nk, pd = ctx.vale_dim, ctx.nk, ctx.pot_dim
    prec = api.PREC_MIXED if args.precision == "mixed" else api.PREC_FP64
    vec = torch.zeros(nk, n, n, dtype=torch.complex128, device="cuda")
    w = ctx.scf_iteration(sysm.pot_coeffs, n, precision=prec, vectors=vec)
    nocc = 2 * len(sysm.site_type) if args.config.startswith("si") else max(1, n // 4)
    occ = np.zeros((nk, n))
    occ[:, :nocc] = 2.0 / nk
    ctx.make_valence_rho(occ, vec, w)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    for _ in range(2):
        tr, en, _ = ctx.make_valence_rho(occ, vec, w)
    dt = (time.perf_counter() - t0) / 2
    torch.cuda.profiler.stop()
    plen = n * (n + 1) // 2
    print(json.dumps({"workload": f"{args.config}, {nk} k (stride {args.k_stride}), {nocc} occupied",
                      "s_per_call": dt, "electrons": float(tr[0, 0]),
                      "trace_bytes_per_launch": nk * plen * 16 * (3 + pd + 1)}), flush=True)


# ---------------------------------------------------------------------------
def clocks_start():
    try:
        f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"
        pr = subprocess.Popen(["nvidia-smi", "-i", dev, f"--query-gpu={q}",
                               "--format=csv,noheader,nounits", "-lms", "200"],
                              stdout=f, stderr=subprocess.DEVNULL)
        return pr, f
    except Exception:
        return None, None


def clocks_stop(pr, f):
    if pr is None:
        return None
    pr.terminate()
    try:
        pr.wait(timeout=5)
    except Exception:
        pr.kill()
    f.flush()
    f.seek(0)
    rows = [r.strip().split(",") for r in f.read().splitlines() if r.strip()]
    f.close()
    os.unlink(f.name)
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for r in rows:
        try:
            sm.append(float(r[1]))
            mx.append(float(r[2]))
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        except (ValueError, IndexError):
            continue
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
            "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def shard(nk, world, rank):
    """Contiguous k-range of a rank (the k-point decomposition of the path)."""
    from olcao_gb300.kshard import shard_range
    return shard_range(nk, world, rank)


# ---------------------------------------------------------------------------
# Largest pencil the CPU legs solve per sample.  LAPACK zhegv with vectors
# costs ~n^3 (measured on the GPU machine's 16 Grace cores: 1.5 / 11.6 / 90.7 s at
# n = 832 / 1664 / 3328, exponent 2.97), so one Si512 k-point (n = 6656) would
# take ~12 min; larger workloads are timed on an n_s x n_s sample and scaled by
# (n / n_s)^3 and the number of k-points.
CPU_SAMPLE_N = 1664
CPU_BUDGET_S = 120.0


def cpu_iteration_sample(H_list, S_list, coeffs_scale=1.0):
    """CPU oracle leg for the sampled k-points: LAPACK zhegv per k (the
    reference's solveZHEGV); returns seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import scipy.linalg as sl
    t0 = time.perf_counter()
    for H, S in zip(H_list, S_list):
        sl.eigh(H * coeffs_scale, S, type=1, driver="gv", lower=False, check_finite=False)
    return time.perf_counter() - t0


def synthetic_pencil(n, seed):
    """Seeded Hermitian H and Hermitian positive definite S of order n: the
    cost of LAPACK zhegv does not depend on the entries beyond its QR
    iteration count."""
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return (A + A.conj().T) / 2, B @ B.conj().T / n + np.eye(n)


def one_thread_zhegv(n):
    """Seconds of one zhegv of order n in a child process limited to one
    BLAS thread (the reference is serial)."""
    code = ("import time, numpy as np, scipy.linalg as sl; rng = np.random.default_rng(7); n = %d; "
            "A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)); H = (A + A.conj().T) / 2; "
            "B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)); "
            "S = B @ B.conj().T / n + np.eye(n); t = time.perf_counter(); "
            "sl.eigh(H, S, type=1, driver='gv', lower=False, check_finite=False); "
            "print(time.perf_counter() - t)" % n)
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1", MKL_NUM_THREADS="1")
    try:
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
        return float(r.stdout.strip().splitlines()[-1])
    except Exception:
        return None


def run_reference(args, world, rank):
    """CPU restatement of the iteration (oracle port): per k, H(k) assembled
    from the packed operators (readPackedMatrixAccum) and LAPACK zhegv
    (solveZHEGV), on a bounded sample of the workload.  The batched workload
    sums the two systems' scaled samples."""
    if rank != 0:
        return
    if args.config != "batched":
        print(json.dumps(reference_line(args, world, args.config)), flush=True)
        return
    lines = [reference_line(args, world, name) for name in BATCHED_PARTS]
    v = sum(l["value"] for l in lines)
    line = dict(lines[0])
    line.update({"value": v, "ms_per_step": v * 1e3, "value_from": "sum of the parts' scaled samples",
                 "steps": min(l["steps"] for l in lines),
                 "data": "synthetic seeded (graphite, si8)",
                 "config": {"workload": WORKLOADS["batched"], "form": "stored", "precision": "fp64"},
                 "cpu_baseline": {"value": v, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                                  "sample": "; ".join(f"{n}: {l['cpu_baseline']['sample']}"
                                                      for n, l in zip(BATCHED_PARTS, lines))},
                 "one_thread": None, "k_solves_per_s": (8192 + 512) / v,
                 "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    print(json.dumps(line), flush=True)


def reference_line(args, world, config):
    """The reference arm's JSON line for one workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from olcao_gb300 import system as S
    full = S.SYSTEMS[config]()
    nk, n, pd = full.num_kpoints, full.vale_dim, full.pot_dim
    t0 = time.perf_counter()
    if n <= CPU_SAMPLE_N:
        # real pencils: the oracle's packed operators of sampled k-points
        ns = max(1, min(args.cpu_sample_k, nk))
        idx = np.linspace(0, nk - 1, ns).round().astype(int)
        part = S.SYSTEMS[config]()
        part.kpoints_abc = full.kpoints_abc[idx]
        o = orc.Oracle(part)
        packed = o.packed_operators()
        n_s, scale = n, nk / ns
        sample = (f"{ns} of {nk} k-points of the oracle's stored operators: assembly + zhegv "
                  f"(n = {n}) per k, scaled by {nk}/{ns}")
    else:
        # seeded synthetic operators of order n_s (the workload's own pencils
        # take hours of CPU integrals to build); zhegv cost ~ n^3
        n_s = CPU_SAMPLE_N
        rng = np.random.default_rng(12)
        plen = n_s * (n_s + 1) // 2
        H, Sm = synthetic_pencil(n_s, 13)
        rows, cols = orc.packed_index(n_s)
        packed = {"S": np.stack([Sm[rows, cols].real, Sm[rows, cols].imag], -1)[None],
                  "KE": np.stack([H[rows, cols].real, H[rows, cols].imag], -1)[None]}
        for name in ["NP"] + [f"V{j}" for j in range(pd)]:
            packed[name] = 1e-3 * rng.standard_normal((1, plen, 2))
        scale = nk * (n / n_s) ** 3
        sample = (f"one k-point sample of order n_s = {n_s} (seeded synthetic packed NP, KE, V_j, S: "
                  f"assembly of {3 + pd} terms + zhegv), scaled by nk (n/n_s)^3 = {nk} x "
                  f"({n}/{n_s})^3 = {scale:.0f} (zhegv cost measured ~n^2.97 on the GPU box's host)")
    t_setup = time.perf_counter() - t0
    # the requested warm-up samples, then the requested timed samples as long
    # as they fit the CPU time budget (a run that hits it reports fewer steps)
    times = []
    for step in range(args.warmup + args.steps):
        c = full.pot_coeffs * (1.0 + 0.01 * ((step % 5) - 2))
        t0 = time.perf_counter()
        hp = orc.assemble(packed, c)
        orc.zhegv(hp, packed["S"], n_s, n_s)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
            if sum(times) > CPU_BUDGET_S:
                break
    t_sample = float(np.mean(times))
    v = t_sample * scale
    n1 = min(n, 832)
    one = one_thread_zhegv(n1)
    one_thread = None
    if one is not None:
        s1 = nk * (n / n1) ** 3
        one_thread = {"value": one * s1, "unit": "s", "cores": 1,
                      "sample": f"one zhegv of order {n1} (seeded synthetic pencil, one BLAS thread), "
                                f"scaled by nk (n/{n1})^3 = {s1:.0f}; assembly excluded"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s",
            "n_gpus": world, "steps": len(times), "warmup": args.warmup, "ms_per_step": t_sample * 1e3,
            "value_from": f"ms_per_step (one timed sample) x {scale:.4g}",
            "steps_requested": args.steps, "warmup_requested": args.warmup,
            "higher_is_better": False, "scaling": "strong",
            "vs_baseline": None, "dtype": "fp64", "data": f"synthetic seeded ({full.name})",
            "config": {"workload": WORKLOADS[config], "form": "stored",
                       "precision": "fp64"},
            "cpu_baseline": {"value": v, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                             "sample": sample},
            "one_thread": one_thread,
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "t_setup_s_sample": t_setup}
    return line


# ---------------------------------------------------------------------------
def run_batched(args):
    """The uneven batch: a mixed pass over graphite's 8192 k (n = 32, the
    in-shared-memory batched solver) and one over Si8's 512 k (n = 104, the
    batched FP32 solver and Rayleigh-Ritz) per step, each replayed as a CUDA
    graph.  Reports s per step and k-point solves per second."""
    import torch
    from olcao_gb300 import api, build
    from olcao_gb300 import system as S
    if not os.path.exists(api.LIB_PATH):
        build.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    parts = []
    for name in BATCHED_PARTS:
        sysm = S.SYSTEMS[name]()
        ctx = api.Context(sysm)
        ctx.scf_prepare(api.PREC_FP64, api.FORM_STORED)
        cs = [sysm.pot_coeffs * (1.0 + 0.01 * ((s % 5) - 2)) for s in range(5)]
        parts.append({"name": name, "ctx": ctx, "coeffs": cs,
                      "dco": [torch.from_numpy(c).cuda() for c in cs],
                      "host": [torch.from_numpy(c).pin_memory() for c in cs],
                      "eig": torch.empty(ctx.nk, ctx.vale_dim, dtype=torch.float64, device="cuda"),
                      "eig_host": torch.empty(ctx.nk, ctx.vale_dim, dtype=torch.float64).pin_memory(),
                      "vec": torch.empty(ctx.nk, ctx.vale_dim, ctx.vale_dim, dtype=torch.complex128,
                                         device="cuda")})

    def step(s, host=False):
        for p in parts:
            c = p["host"][s % 5].numpy() if host else p["dco"][s % 5]
            out = p["eig_host"].numpy() if host else p["eig"]
            p["ctx"].scf_iteration(c, p["ctx"].vale_dim, eig_out=out, vectors=p["vec"],
                                   precision=api.PREC_MIXED, graph=True)

    for w in range(args.warmup):
        step(w)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = api.launch_count()
    pr, fh = clocks_start()
    torch.cuda.synchronize()
    ev0.record(stream)
    for s in range(args.steps):
        step(s)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = clocks_stop(pr, fh)
    launches = api.launch_count() - l0
    ms = ev0.elapsed_time(ev1) / args.steps
    mixed = [p["eig"].cpu().numpy().copy() for p in parts]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 5))
    for s in range(e2e_steps):
        step(s, host=True)
    torch.cuda.synchronize()
    e2e = (time.perf_counter() - t0) / e2e_steps
    acc = {}
    last = (args.steps - 1) % 5
    for p, wm in zip(parts, mixed):
        w64 = p["ctx"].scf_iteration(p["dco"][last], p["ctx"].vale_dim, precision=api.PREC_FP64)
        acc[p["name"]] = float(np.abs(wm - w64).max())
    nk_total = sum(p["ctx"].nk for p in parts)
    h2d = sum(p["host"][0].numel() * 8 for p in parts)
    d2h = sum(p["eig_host"].numel() * 8 for p in parts)
    line = {"metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "strong",
            "vs_baseline": None, "dtype": "fp64+fp32+bf16", "data": "synthetic seeded (graphite, si8)",
            "config": {"workload": WORKLOADS["batched"], "form": "stored", "precision": "mixed",
                       "num_kpoints": nk_total, "cuda_graph": True},
            "k_solves_per_s": nk_total / (ms / 1e3),
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps},
            "gpu_launches": int(launches),
            "accuracy": {"max_abs_eig_err_ha": acc,
                         "reference": "plain FP64 GPU path on the same H(k), S(k)"},
            "roofline": None, "cpu_baseline": None, "clocks": clocks}
    print(json.dumps(line), flush=True)
    for p in parts:
        p["ctx"].close()


# ---------------------------------------------------------------------------
def run_ours(args, world, rank, dist):
    import torch
    from olcao_gb300 import api, build
    from olcao_gb300 import system as S

    if not os.path.exists(api.LIB_PATH):
        build.build()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    full = S.SYSTEMS[args.config]()
    if args.nk > 0:
        full.kpoints_abc = full.kpoints_abc[:args.nk]
    nk_total = full.num_kpoints
    lo, hi = shard(nk_total, world, rank)
    sysm = full
    if world > 1:
        sysm.kpoints_abc = full.kpoints_abc[lo:hi]
    stream = torch.cuda.current_stream()
    ctx = api.Context(sysm)
    n, nk, pd = ctx.vale_dim, ctx.nk, ctx.pot_dim
    nstates = n
    form = api.FORM_STORED if args.form == "stored" else api.FORM_FUSED
    prec = api.PREC_MIXED if args.precision == "mixed" else api.PREC_FP64

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    ctx.scf_prepare(api.PREC_FP64, form)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_setup = ev0.elapsed_time(ev1) / 1e3

    coeff_steps = [full.pot_coeffs * (1.0 + 0.01 * ((s % 5) - 2)) for s in range(5)]
    dco = [torch.from_numpy(c).cuda() for c in coeff_steps]
    eig = torch.empty(nk, nstates, dtype=torch.float64, device="cuda")
    # eigenvectors are produced every step, as solveZHEGV does for the density
    vec = torch.empty(nk, nstates, n, dtype=torch.complex128, device="cuda")
    graph = not args.no_graph
    for w in range(args.warmup):
        ctx.scf_iteration(dco[w % 5], nstates, eig_out=eig, vectors=vec, precision=prec, graph=graph)
    torch.cuda.synchronize()
    # under `ncu --profile-from-start off` only the timed steps are captured
    mark = os.environ.get("OLC_BENCH_PROFILE_TIMED") == "1"

    # ---- timed region: device-resident inputs ---------------------------------
    l0 = api.launch_count()
    pr, fh = clocks_start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if mark:
        torch.cuda.profiler.start()
    ev0.record(stream)
    for s in range(args.steps):
        ctx.scf_iteration(dco[s % 5], nstates, eig_out=eig, vectors=vec, precision=prec, graph=graph)
    ev1.record(stream)
    torch.cuda.synchronize()
    if mark:
        torch.cuda.profiler.stop()
    if dist:
        dist.barrier()
    clocks = clocks_stop(pr, fh)
    launches = api.launch_count() - l0
    ms = ev0.elapsed_time(ev1) / args.steps
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    eig_main = eig.cpu().numpy().copy()

    # ---- e2e: public API with host buffers ------------------------------------
    host_c = [torch.from_numpy(c).pin_memory() for c in coeff_steps]
    eig_host = torch.empty(nk, nstates, dtype=torch.float64).pin_memory()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        ctx.scf_iteration(host_c[s % 5].numpy(), nstates, eig_out=eig_host.numpy(),
                          vectors=vec, precision=prec, graph=graph)
    torch.cuda.synchronize()
    e2e = (time.perf_counter() - t0) / e2e_steps

    # ---- stage breakdown: profiled passes launched directly -------------------
    ctx.profile(True)
    ctx.profile_reset()
    nprof = 2
    for s in range(nprof):
        ctx.scf_iteration(dco[s % 5], nstates, eig_out=eig, vectors=vec, precision=prec)
    prof = ctx.profile_read()
    work = ctx.profile_work()
    ctx.profile(False)
    if dist:
        t = torch.tensor([e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e = float(t.item())

    # ---- next stage: valence density + traces of the last step's vectors ------
    vrho = None
    if rank == 0:
        nocc_v = 2 * len(full.site_type) if args.config.startswith("si") else max(1, nstates // 4)
        occ = np.zeros((nk, nstates))
        occ[:, :nocc_v] = 2.0 / nk_total
        eh = eig.cpu().numpy()
        ctx.make_valence_rho(occ, vec, eh)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 3
        for r in range(reps):
            tr_v, en_v, _ = ctx.make_valence_rho(occ, vec, eh)
        vrho = {"s_per_call": (time.perf_counter() - t0) / reps, "occupied_states": nocc_v,
                "operators_traced": 3 + pd,
                "operator_bytes_read": nk * (3 + pd) * (n * (n + 1) // 2) * 16,
                "electrons": float(tr_v[0, 0]), "electron_energy_ha": float(en_v[0]),
                "note": "makeValenceRho: rho = X diag(f) X^H (split-BF16, FP64-accurate) "
                        "and its traces with S, NP, KE, V_j; not part of the timed step"}

    # ---- plain FP64 GPU path on the same step (accuracy and speed-up) ---------
    t_fp64 = None
    acc = None
    if prec == api.PREC_MIXED and world == 1 and not args.no_fp64:
        last = (args.steps - 1) % 5
        # one pass with the same inputs as the last timed step (its workspace
        # set-up is a small part of a pass of this size)
        torch.cuda.synchronize()
        ev0.record(stream)
        ctx.scf_iteration(dco[last], nstates, eig_out=eig, vectors=vec, precision=api.PREC_FP64)
        ev1.record(stream)
        torch.cuda.synchronize()
        t_fp64 = ev0.elapsed_time(ev1) / 1e3
        w64 = eig.cpu().numpy()
        nocc = 2 * len(full.site_type) if args.config.startswith("si") else min(nstates, 4 * len(full.site_type) // 2)
        band = lambda w: float(2.0 * w[:, :nocc].sum() / w.shape[0])
        acc = {"max_abs_eig_err_ha": float(np.abs(eig_main - w64).max()),
               "band_energy_err_ha": abs(band(eig_main) - band(w64)),
               "reference": "plain FP64 GPU path (cuSOLVER zhegvd) on the same H(k), S(k)"}

    # ---- fused form (integrals recomputed with the coefficients) --------------
    t_fused = None
    if rank == 0 and not args.no_fused and world == 1:
        ctxf = api.Context(sysm)
        ctxf.scf_prepare(api.PREC_FP64, api.FORM_FUSED)
        ctxf.scf_iteration(dco[0], nstates, eig_out=eig, vectors=vec, precision=prec)
        torch.cuda.synchronize()
        ev0.record(stream)
        ctxf.scf_iteration(dco[1], nstates, eig_out=eig, vectors=vec, precision=prec)
        ev1.record(stream)
        torch.cuda.synchronize()
        t_fused = ev0.elapsed_time(ev1) / 1e3
        ctxf.close()

    if rank != 0:
        return
    # ---- per-stage rooflines; the dominant kernel's goes into `roofline` ------
    peaks, peak_kind = measured_peaks()
    hbm = peaks["hbm_gbs"]
    tc_peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
    step_ms = ms
    plen = n * (n + 1) // 2
    asm_bytes = nk * ((2 + pd) * plen * 16 + n * n * 16)
    kernels = {
        # stage: (kernel, bound)
        "tridiag": ("hetrd_panel_kernel + tc_gemm_kernel<f32> trailing updates (blocked FP32 "
                    "tridiagonalisation, one cluster per k)", "hbm"),
        "split": ("tc_gemm_kernel<fixed> (tcgen05 8-bit split-digit products, FP64-accurate) + digit slicing",
                  "tensor"),
        "backtransform": ("tc_gemm_kernel<f32> (tcgen05 compact-WY back-transform, X = U^-1 Z)", "tensor"),
        "assemble": ("assemble_full_kernel (H(k) from the resident packed operators)", "hbm"),
    }
    stage_roof = {}
    for st, (kname, bound) in kernels.items():
        launches_s, ms_s = prof[st]
        fl, by = work[st]
        if st == "assemble":
            by = asm_bytes * nprof
        if ms_s <= 0:
            continue
        sec = ms_s / 1e3
        if bound == "hbm":
            ach = by / sec / 1e9
            row = {"kernel": kname, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                   "frac": ach / hbm, "algorithmic_bytes_per_step": by / nprof}
        else:
            ach = fl / sec / 1e12
            row = {"kernel": kname, "bound": "tensor", "achieved": ach, "peak": tc_peak,
                   "unit": "TFLOP/s", "frac": ach / tc_peak if tc_peak else None,
                   "tensor_flops_per_step": fl / nprof}
        row["ms_per_step"] = ms_s / nprof
        row["share_of_step"] = (ms_s / nprof) / step_ms
        row["launches_per_step"] = launches_s / nprof
        stage_roof[st] = row
    dom = max(stage_roof, key=lambda k: stage_roof[k]["ms_per_step"])
    d = stage_roof[dom]
    roof = {"kernel": d["kernel"], "bound": d["bound"], "achieved": d["achieved"], "peak": d["peak"],
            "unit": d["unit"], "frac": d["frac"], "traffic": None,
            "peak_source": f"{peak_kind} ({'HBM copy' if d['bound'] == 'hbm' else 'sustained cuBLAS bf16'})",
            "stage": dom, "share_of_step": d["share_of_step"],
            "launch_ms": d["ms_per_step"] / max(1.0, d["launches_per_step"])}
    # the whole solve against the sustained tensor peak, counting the
    # generalised eigen-solve as 23 n^3 real flops per k (LAWN-41 style)
    solve_frac = {"flops_per_step": 23.0 * n ** 3 * nk,
                  "achieved_tflops": 23.0 * n ** 3 * nk / (step_ms / 1e3) / 1e12,
                  "frac_of_sustained_bf16": (23.0 * n ** 3 * nk / (step_ms / 1e3) / 1e12) / tc_peak
                  if tc_peak else None}

    # ---- CPU baseline (oracle leg) on a bounded sample -------------------------
    cpu = None
    if not args.no_cpu and world == 1:
        if n <= CPU_SAMPLE_N:
            ns = max(1, min(args.cpu_sample_k, nk))
            ks = np.linspace(0, nk - 1, ns).round().astype(int)
            Hs, Ss = [], []
            for k in ks:
                H, Sm = ctx.scf_matrices(coeff_steps[0], int(k))
                Hs.append(H)
                Ss.append(Sm)
            dt = cpu_iteration_sample(Hs, Ss)
            cpu = {"value": dt * nk / ns, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"LAPACK zhegv on {ns} of {nk} k-points of this H(k), S(k), "
                             f"scaled by {nk}/{ns} (assembly excluded)"}
        else:
            # the leading n_s x n_s block of this workload's H(Gamma), S(Gamma)
            H, Sm = ctx.scf_matrices(coeff_steps[0], 0)
            n_s = CPU_SAMPLE_N
            Hb, Sb = H[:n_s, :n_s].copy(), Sm[:n_s, :n_s].copy()
            del H, Sm
            cpu_iteration_sample([Hb[:256, :256]], [Sb[:256, :256]])     # BLAS threads up
            dt = cpu_iteration_sample([Hb], [Sb])
            sc = nk * (n / n_s) ** 3
            cpu = {"value": dt * sc, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"LAPACK zhegv on the leading {n_s} x {n_s} block of this H(Gamma), "
                             f"S(Gamma), {dt:.1f} s, scaled by nk (n/n_s)^3 = {sc:.0f} "
                             f"(assembly excluded)"}

    stages = {k: {"launches_per_step": v[0] / nprof, "ms_per_step": v[1] / nprof}
              for k, v in prof.items()}
    line = {"metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": False, "scaling": "strong", "vs_baseline": None,
            "dtype": "fp64+fp32+bf16" if prec == api.PREC_MIXED else "fp64",
            "data": f"synthetic seeded ({full.name}, seed {full.seed})",
            "config": {"workload": WORKLOADS[args.config], "form": args.form,
                       "precision": ("mixed: FP32 solve + split-BF16 Rayleigh-Ritz, FP64 integrals"
                                     if prec == api.PREC_MIXED else "fp64 (plain path)"),
                       "n_basis": n,
                       "num_kpoints": nk_total, "pot_dim": pd,
                       "l2": "resident integrals larger than L2, no flush",
                       "cuda_graph": graph and prec == api.PREC_MIXED and args.form == "stored"},
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": pd * 8,
                    "d2h_bytes_per_step": nk * nstates * 8, "steps": e2e_steps},
            "gpu_launches": int(launches),
            "roofline": roof, "stage_rooflines": stage_roof, "solve_23n3": solve_frac,
            "cpu_baseline": cpu, "clocks": clocks,
            "t_setup_s": t_setup, "t_iter_fused_s": t_fused,
            "t_iter_fp64_gpu_s": t_fp64,
            "speedup_vs_fp64_gpu": (t_fp64 / (ms / 1e3)) if t_fp64 else None,
            "accuracy": acc,
            "valence_rho": vrho,
            "stages": stages}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        td.init_process_group(backend)
        dist = td
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.valence_rho_only:
        run_valence_rho_only(args)
    elif args.config == "batched":
        if rank == 0:
            run_batched(args)
    else:
        run_ours(args, world, rank, dist)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
