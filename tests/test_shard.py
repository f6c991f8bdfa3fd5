"""CPU checks of the multi-GPU sharding logic (segment-tree-based-clipping_gb300/
shard.py): the longest-processing-time partition of one batched job, the
sampled-K cost estimate, and the host-side gather of per-pair outputs over a
world_size-2 gloo group.  The per-pair clip inside the ranks is the oracle, a
CPU stand-in for the GPU call (test only): what is checked is that every pair
is clipped exactly once and that the gathered job equals the single-rank
job."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

import shard
import sbclip_gen as gen


def test_lpt_covers_every_pair_once_and_balances():
    rng = np.random.default_rng(1)
    nb = np.exp(rng.uniform(np.log(3), np.log(2049), 5000)).astype(int)
    nc = np.exp(rng.uniform(np.log(3), np.log(2049), 5000)).astype(int)
    costs = shard.pair_costs(nb, nc)
    for world in (1, 2, 3, 8):
        parts = shard.lpt_partition(costs, world)
        allidx = np.concatenate(parts)
        assert len(allidx) == len(costs) and np.array_equal(np.sort(allidx), np.arange(len(costs)))
        for p in parts:
            assert np.all(np.diff(p) > 0)  # job order within a rank
        ld = shard.loads(costs, parts)
        assert ld.max() <= shard.lpt_bound(costs, world) + 1e-6
        assert ld.max() / ld.mean() < 1.01  # many small pairs: near-perfect balance


def test_lpt_with_a_few_dominant_pairs():
    """The large pairs of the uneven workload (16 of 200k vertices among many
    small ones) land on different ranks before the small ones fill in."""
    costs = np.concatenate([shard.pair_costs([200_000] * 16, [200_000] * 16),
                            shard.pair_costs(np.full(20000, 300), np.full(20000, 300))])
    parts = shard.lpt_partition(costs, 8)
    big_per_rank = [int((p < 16).sum()) for p in parts]
    assert big_per_rank == [2] * 8
    ld = shard.loads(costs, parts)
    assert ld.max() / ld.mean() < 1.02


def test_sampled_hits_per_size_class():
    n = np.array([10, 12, 100, 120, 1000, 1020, 5000])
    est = shard.estimate_hits(n, [0, 2, 4], [5.0, 50.0, 500.0])
    assert list(est[:6]) == [5.0, 5.0, 50.0, 50.0, 500.0, 500.0]
    assert est[6] == pytest.approx(185.0)  # class not sampled: overall mean


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _job():
    pairs = gen.small_pairs(48, seed=4321)
    nb = np.array([len(b) for b, _ in pairs])
    nc = np.array([len(c) for _, c in pairs])
    return pairs, nb, nc


def _clip(pair):
    import oracle_py as O
    b, c = pair
    return [r.copy() for r in O.rings_of(O.clip(b, [c])["overlays"][0])]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        pairs, nb, nc = _job()
        # sampled K: the intersection counts of every 6th pair (the same on every rank)
        import oracle_py as O
        sample = np.arange(0, len(pairs), 6)
        hits = [len(O.clip(pairs[i][0], [pairs[i][1]])["overlays"][0]["uniq_b"]) for i in sample]
        costs = shard.pair_costs(nb, nc, shard.estimate_hits(nb + nc, sample, hits))
        parts = shard.lpt_partition(costs, world)
        local = {int(i): _clip(pairs[i]) for i in parts[rank]}
        got = shard.gather_outputs(local, len(pairs))
        if rank == 0:
            assert got is not None and len(got) == len(pairs)
            for i, pr in enumerate(pairs):
                want = _clip(pr)
                assert len(got[i]) == len(want)
                assert all(np.array_equal(x, y) for x, y in zip(got[i], want)), i
            summary = shard.shard_summary(costs, parts)
            with open(os.path.join(out_dir, "ok"), "w") as f:
                f.write(repr(summary))
        else:
            assert got is None
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_job_equals_single_rank(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    text = (tmp_path / "ok").read_text()
    assert "'ranks': 2" in text
