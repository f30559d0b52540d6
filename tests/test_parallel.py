"""Row sharding of a product across ranks (the multi-GPU path), on CPU with
gloo and world size 2: segment shards balanced by panel values cover every row
once, each rank's rows computed by the plan executor alone add up (all_reduce)
to the full product exactly, and the step-time reduction takes the maximum."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from hierarchicalmatrices import Plan, parallel  # noqa: E402
from oracle import oracle as O  # noqa: E402
from plan_emulator import emulate  # noqa: E402


def test_balanced_ranges():
    w = np.array([5, 1, 1, 1, 1, 1, 5, 0, 2], dtype=float)
    for parts in (1, 2, 3, 4, 12):
        cuts = parallel.balanced_ranges(w, parts)
        assert cuts[0] == 0 and cuts[-1] == len(w) and np.all(np.diff(cuts) >= 0) and len(cuts) == parts + 1
    cuts = parallel.balanced_ranges(np.ones(100), 4)
    assert list(cuts) == [0, 25, 50, 75, 100]
    with pytest.raises(ValueError):
        parallel.balanced_ranges([1.0, -1.0], 2)


def test_segment_shards_cover_rows_once():
    x, y = O.beta_points(8192, 3)
    P = Plan(x, y, 1.0, 0.0, 1.0, 0.0)
    for world in (1, 2, 3, 8):
        shards = parallel.segment_shards(P, world)
        rows = np.concatenate([s["rows"] for s in shards])
        assert np.array_equal(np.sort(rows), np.arange(8192))
        lo = [s["segments"][0] for s in shards]
        assert lo == sorted(lo)
    inst = parallel.instance_shards([1024, 65536, 2048, 4096], 2)
    assert inst[0][0] == 0 and inst[-1][1] == 4 and inst[0][1] == inst[1][0]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, n, out_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x, y = O.beta_points(n, 5)
        P = Plan(x, y, 1.0, 0.0, 1.0, 0.0)
        b = np.random.default_rng(1).standard_normal(n)
        shard = parallel.segment_shards(P, world)[rank]
        part = torch.tensor(emulate(P, O.CAUCHY, b, segments=shard["segments"]))
        dist.all_reduce(part, op=dist.ReduceOp.SUM)
        slowest = parallel.max_over_ranks(1.0 + rank)
        if rank == 0:
            full = emulate(P, O.CAUCHY, b)
            np.savez(out_path, assembled=part.numpy(), full=full, slowest=slowest)
    finally:
        dist.destroy_process_group()


def test_row_sharded_product_gloo(tmp_path):
    n, world = 4096, 2
    out = str(tmp_path / "sharded.npz")
    mp.spawn(_rank_main, args=(world, _free_port(), n, out), nprocs=world, join=True)
    r = np.load(out)
    assert np.array_equal(r["assembled"], r["full"])        # every row from exactly one rank
    assert float(r["slowest"]) == 2.0
