"""Sharding one batched clipping job over several GPUs (one process per GPU).

A single pair does not shard: its segment tree and its ring tracing are
global.  The batched workloads do: the pairs of a many-pair batch, and the
overlays of one base against many overlays (the base replicated on every
rank), are independent.  The reference has no multi-GPU code; its one-to-many
driver clips overlay after overlay (src/clip.cpp:1702-2062), and that loop is
what is partitioned here.

* cost of a pair: n log2 n for its n = n_base + n_overlay edges (the tree
  build and the sorts), plus its intersection count K (the merge, labelling
  and tracing rows), with K estimated per size class from a sampled subset of
  pairs clipped beforehand;
* partition: greedy longest processing time first (each pair, most costly
  first, to the least loaded rank), whose largest load is within 4/3 of the
  optimum; each rank keeps its pairs in job order;
* exchange: none during the job.  Per-pair outputs are gathered on rank 0 by
  the host afterwards (a gloo group: no device collective on the data path).
"""
from __future__ import annotations

import heapq

import numpy as np


def pair_costs(n_base, n_overlay, hits=None, hit_weight: float = 1.0) -> np.ndarray:
    """Estimated cost of every pair: n log2 n + hit_weight * K."""
    n = np.asarray(n_base, np.float64) + np.asarray(n_overlay, np.float64)
    cost = n * np.log2(np.maximum(n, 2.0))
    if hits is not None:
        cost = cost + hit_weight * np.asarray(hits, np.float64)
    return cost


def size_class(n) -> np.ndarray:
    """Size class of a pair of n edges: floor(log2 n)."""
    return np.floor(np.log2(np.maximum(np.asarray(n, np.float64), 1.0))).astype(np.int64)


def estimate_hits(n_pairs_edges, sample_idx, sample_hits) -> np.ndarray:
    """K for every pair: the mean K of the sampled pairs of its size class
    (the overall sample mean for a class the sample missed)."""
    cls = size_class(n_pairs_edges)
    sample_idx = np.asarray(sample_idx, np.int64)
    sample_hits = np.asarray(sample_hits, np.float64)
    est = np.full(len(cls), float(sample_hits.mean()) if len(sample_hits) else 0.0)
    if len(sample_idx):
        scls = cls[sample_idx]
        for c in np.unique(scls):
            est[cls == c] = sample_hits[scls == c].mean()
    return est


def lpt_partition(costs, world: int) -> list[np.ndarray]:
    """Greedy longest-processing-time partition of the pairs over `world`
    ranks; each rank's pair indices in ascending (job) order."""
    costs = np.asarray(costs, np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    order = np.argsort(-costs, kind="stable")
    heap = [(0.0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def loads(costs, parts) -> np.ndarray:
    costs = np.asarray(costs, np.float64)
    return np.array([costs[p].sum() for p in parts])


def lpt_bound(costs, world: int) -> float:
    """An upper bound on LPT's largest load: the mean load plus the largest
    single cost (every pair is placed on a rank whose load was at most the
    mean when it was placed)."""
    costs = np.asarray(costs, np.float64)
    if not len(costs):
        return 0.0
    return float(costs.sum() / world + costs.max())


def gather_outputs(local: dict, n_total: int, group=None):
    """Gather {pair index: output} from every rank onto rank 0 over the host
    (gather_object on `group`, e.g. a gloo group).  Rank 0 gets the outputs in
    job order (a list of n_total); other ranks get None.  Raises if a pair is
    missing or was produced twice."""
    import torch.distributed as dist

    rank = dist.get_rank()
    world = dist.get_world_size()
    objs = [None] * world if rank == 0 else None
    dist.gather_object(local, objs, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * n_total
    seen = np.zeros(n_total, bool)
    for part in objs:
        for i, v in part.items():
            if seen[i]:
                raise RuntimeError(f"pair {i} produced by two ranks")
            seen[i] = True
            out[i] = v
    if not seen.all():
        raise RuntimeError(f"{int((~seen).sum())} pairs missing from the gather")
    return out


def shard_summary(costs, parts) -> dict:
    ld = loads(costs, parts)
    mean = float(ld.mean()) if len(ld) else 0.0
    return {"ranks": len(parts), "pairs_per_rank": [int(len(p)) for p in parts],
            "max_over_mean_load": float(ld.max() / mean) if mean > 0 else 1.0}


__all__ = ["pair_costs", "size_class", "estimate_hits", "lpt_partition", "loads", "lpt_bound",
           "gather_outputs", "shard_summary"]
