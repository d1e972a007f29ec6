"""Multi-GPU host logic on CPU ranks (gloo, world_size 2).

The path shards by photons: rank r simulates its own contiguous photon range and the field is
one sum at the end (MCX's own design, src/mcx_core.cu:3007, 3748-3759).  Per-photon seeding
makes the union of the ranks' photons exactly the single-rank photon set, so two CPU ranks
running the oracle on their halves and reducing must equal one rank running everything.
"""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def shard(nphoton: int, world: int, rank: int) -> tuple[int, int]:
    """Photon range [offset, offset + n) of `rank` (the remainder goes to the first ranks)."""
    base, odd = divmod(nphoton, world)
    n = base + (1 if rank < odd else 0)
    offset = rank * base + min(rank, odd)
    return offset, n


def test_shards_partition_the_photons():
    for total in (0, 1, 7, 1000, 1_000_003):
        for world in (1, 2, 3, 8):
            ranges = [shard(total, world, r) for r in range(world)]
            assert sum(n for _, n in ranges) == total
            pos = 0
            for off, n in ranges:
                assert off == pos
                pos += n


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, nphoton: int, out_path: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import mcx_gb300
    from mcx_gb300 import problems
    from oracle import oracle

    pc = mcx_gb300.prepare(problems.workload0(nphoton, seed=99))
    off, n = shard(nphoton, world, rank)
    r = oracle.run(pc, nphoton=n, photon_offset=off, threads=2)
    raw = torch.from_numpy(r["raw"].ravel(order="F").copy())
    e = torch.tensor([r["stat"]["e_launch"], r["stat"]["e_absdep"], float(r["stat"]["n_photon"])], dtype=torch.float64)
    dist.all_reduce(raw)
    dist.all_reduce(e)
    if rank == 0:
        np.save(out_path, np.concatenate([raw.numpy(), e.numpy()]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_equal_one(tmp_path, built):
    import mcx_gb300
    from mcx_gb300 import problems
    from oracle import oracle

    nphoton = 20000
    out = tmp_path / "reduced.npy"
    mp.start_processes(_worker, args=(2, _free_port(), nphoton, str(out)), nprocs=2, start_method="spawn")
    red = np.load(out)
    pc = mcx_gb300.prepare(problems.workload0(nphoton, seed=99))
    one = oracle.run(pc, nphoton=nphoton, threads=4)
    raw1 = one["raw"].ravel(order="F")
    nvox = raw1.size
    # same photons, FP64 sums in another order
    assert np.allclose(red[:nvox], raw1, rtol=1e-9, atol=1e-9)
    assert red[nvox + 2] == nphoton
    assert abs(red[nvox] - one["stat"]["e_launch"]) < 1e-6
    assert abs(red[nvox + 1] - one["stat"]["e_absdep"]) / one["stat"]["e_absdep"] < 1e-9
