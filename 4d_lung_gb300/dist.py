"""Multi-GPU layout of the batched 4D reconstruction: respiratory bins are
independent CG solves, so N GPUs run N replicas, each solving a subset of
the bins with no exchange on the data path.  Bins are assigned greedily by
sample count (largest first to the least-loaded rank) so that the ranks'
work is balanced despite the uneven bin occupancy."""
from __future__ import annotations

import numpy as np


def partition_bins(sizes, world_size):
    """Returns one list of bin indices per rank (each list sorted)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    load = np.zeros(world_size, np.int64)
    parts = [[] for _ in range(world_size)]
    for b in np.argsort(-sizes, kind="stable"):
        r = int(np.argmin(load))
        parts[r].append(int(b))
        load[r] += sizes[b]
    return [sorted(p) for p in parts]
