"""Multi-process helpers for products on several GPUs of one node.

The product shards naturally by rows: every row segment's output rows are
written by that segment alone, so contiguous runs of segments (balanced by the
panel bytes they stream) can go to different ranks with no reduction of y;
each rank needs all of x (one all-gather per product when x is itself
sharded).  Independent matrices (a batch of instances) shard the same way by
instance.  Ranks are one process per GPU (torchrun), read from the
environment; collectives go through torch.distributed (NCCL between GPUs,
gloo on the host).
"""
import os

import numpy as np


def rank_info():
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def balanced_ranges(weights, parts):
    """Cuts the sequence of non-negative `weights` into `parts` contiguous
    ranges [lo, hi) of about equal total weight (empty ranges when there are
    fewer items than parts).  Returns a (parts + 1)-array of cut points."""
    w = np.asarray(weights, dtype=np.float64)
    if parts < 1:
        raise ValueError("parts must be >= 1")
    if w.size and w.min() < 0:
        raise ValueError("weights must be non-negative")
    pre = np.concatenate([[0.0], np.cumsum(w)])
    cuts = np.searchsorted(pre, pre[-1] * np.arange(parts + 1) / parts, side="left")
    cuts[0], cuts[-1] = 0, w.size
    return np.maximum.accumulate(np.minimum(cuts, w.size))


def segment_shards(plan, world):
    """Row shards of a product: for each rank, the range of row segments it
    computes and the output rows they cover, balanced by panel values
    (rows x columns of each segment).  `plan` is a hierarchicalmatrices Plan."""
    segs = plan.table("segs")
    weights = segs["nrows"].astype(np.float64) * np.maximum(segs["width"], 1)
    cuts = balanced_ranges(weights, world)
    shards = []
    for r in range(world):
        lo, hi = int(cuts[r]), int(cuts[r + 1])
        rows = segs["row0"][lo:hi], segs["row0"][lo:hi] + segs["nrows"][lo:hi]
        shards.append({"segments": (lo, hi),
                       "rows": np.concatenate([np.arange(a, b) for a, b in zip(*rows)]) if hi > lo
                       else np.zeros(0, dtype=np.int64)})
    return shards


def instance_shards(sizes, world):
    """Instance ranges of a batch for each rank, balanced by instance size."""
    cuts = balanced_ranges(sizes, world)
    return [(int(cuts[r]), int(cuts[r + 1])) for r in range(world)]


def max_over_ranks(value, group=None):
    """The largest of a per-rank float (a step time) over all ranks; the value
    itself when torch.distributed is not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
