"""k-point decomposition of the SCF pass over ranks (one GPU per rank).

Every k-point has its own Bloch sum, orthogonalisation and eigen-solve, so
the pass shards into contiguous k-ranges with no exchange inside it.  An SCF
iteration exchanges only a few KB: the potential coefficients every rank
uses (a broadcast) and the eigenvalues that the occupation step needs for
the Fermi level and the band energy (a gather; the reference sums its
k-point contributions in valeCharge.F90:390-395 and populates states over
all k in populate.F90:172-415).  Uneven k-counts are spread so that shard
sizes differ by at most one.
"""

from __future__ import annotations

import copy
from typing import Tuple

import numpy as np


def shard_range(nk: int, world: int, rank: int) -> Tuple[int, int]:
    """[lo, hi) of the k-points rank `rank` of `world` owns."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(nk, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_system(system, world: int, rank: int):
    """Copy of `system` restricted to this rank's k-range."""
    lo, hi = shard_range(system.num_kpoints, world, rank)
    part = copy.copy(system)
    part.kpoints_abc = np.ascontiguousarray(system.kpoints_abc[lo:hi])
    return part


def broadcast_coefficients(coeffs: np.ndarray, src: int = 0) -> np.ndarray:
    """Every rank gets rank `src`'s potential coefficients."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(coeffs, np.float64)).clone()
    dist.broadcast(t, src)
    return t.numpy()


def gather_eigenvalues(local: np.ndarray, nk_total: int) -> np.ndarray:
    """All ranks' eigenvalues [nk_local, num_states] -> [nk_total, num_states]
    on every rank, in global k order (ranks pad to the largest shard)."""
    import torch
    import torch.distributed as dist
    world, rank = dist.get_world_size(), dist.get_rank()
    ns = local.shape[1]
    size = max(hi - lo for lo, hi in (shard_range(nk_total, world, r) for r in range(world)))
    buf = torch.zeros(size, ns, dtype=torch.float64)
    buf[:local.shape[0]] = torch.from_numpy(np.ascontiguousarray(local, np.float64))
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    out = np.empty((nk_total, ns))
    for r in range(world):
        lo, hi = shard_range(nk_total, world, r)
        out[lo:hi] = parts[r][:hi - lo].numpy()
    return out


def band_energy(local: np.ndarray, nk_total: int, num_occupied: int,
                occupation: float = 2.0) -> float:
    """sum_k w_k sum_{n < num_occupied} e_nk with equal weights 1/nk over the
    whole mesh and fixed (insulator) occupations, summed over ranks."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([occupation * float(local[:, :num_occupied].sum()) / nk_total],
                     dtype=torch.float64)
    dist.all_reduce(t)
    return float(t.item())
