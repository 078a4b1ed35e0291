"""k-point sharding of the SCF pass, with CPU ranks (gloo, world size 2).

The per-k work is the oracle's (CPU) secular equation, standing in for a
GPU rank; the test checks the decomposition and the iteration's exchanges:
coefficient broadcast, eigenvalue gather and band-energy reduction give the
same results as one rank doing every k.
"""

import os
import socket

import numpy as np
import pytest

import oracle as orc
from olcao_gb300 import kshard
from olcao_gb300 import system as S


@pytest.mark.parametrize("nk,world", [(8, 2), (7, 2), (5, 3), (1, 1), (3, 4)])
def test_shard_ranges_cover_the_mesh(nk, world):
    spans = [kshard.shard_range(nk, world, r) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == nk
    for (a, b), (c, d) in zip(spans, spans[1:]):
        assert b == c
    sizes = [b - a for a, b in spans]
    assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    full = S.small_test_system("si2", nk=(3, 1, 1))
    coeffs = full.pot_coeffs * (1.5 if rank == 0 else 0.0)   # only rank 0's are right
    coeffs = kshard.broadcast_coefficients(coeffs)
    part = kshard.shard_system(full, world, rank)
    o = orc.Oracle(part)
    packed = o.packed_operators()
    w, _ = orc.zhegv(orc.assemble(packed, coeffs), packed["S"], o.vale_dim, o.vale_dim)
    allw = kshard.gather_eigenvalues(w, full.num_kpoints)
    eb = kshard.band_energy(w, full.num_kpoints, 4)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([allw.ravel(), [eb]]))
    dist.destroy_process_group()


def test_two_cpu_ranks_match_one_rank(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    full = S.small_test_system("si2", nk=(3, 1, 1))
    o = orc.Oracle(full)
    packed = o.packed_operators()
    coeffs = full.pot_coeffs * 1.5
    w, _ = orc.zhegv(orc.assemble(packed, coeffs), packed["S"], o.vale_dim, o.vale_dim)
    eb = 2.0 * w[:, :4].sum() / full.num_kpoints
    for r in range(world):
        got = np.load(tmp_path / f"rank{r}.npy")
        assert np.abs(got[:-1].reshape(w.shape) - w).max() <= 1e-12
        assert abs(got[-1] - eb) <= 1e-12
