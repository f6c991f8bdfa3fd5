#!/usr/bin/env python3
"""Benchmark: milliseconds per 1M x 1M polygon clip on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload pair_1m_1m|pair_200k_200k|pair_10k_8k|small_pairs_65536|
                                one_to_many_200k_10000]

A step is one full clip of the workload pair (segment tree build, candidate
stab queries, FP64 intersection, merge, labelling and ring tracing) by the
CUDA library.  `value` times K steps on device-resident inputs with CUDA
events on the library's stream; L2 is flushed (a 256 MiB write) between
steps, outside the timed window.  Per-kernel times (the `roofline` and
`kernels_top` entries) come from one extra step outside the timed window,
with every launch bracketed by CUDA events.  `e2e` times the public host API
(sbc_clip_pair): host->device copy of the inputs and the device->host copy of
the result rings (offsets + vertices, into the context's host result memory
that a C caller reads in place) inside every step.

The default line also carries `batched`, the second half of the headline
metric measured in the same run: the 65,536 small pairs (area forward +
backward as one CUDA graph launch per step) and one 200k-vertex base against
10,000 overlays (forward, and area forward + backward), each next to the plain
per-pair GPU path on the same inputs (`--no-batched` leaves it out).  Its
`cpu_baseline.others` adds the reference's CPU build at one thread and at all
host threads on the 10k x 8k pair and Foster's sequential code (the
reference's own baseline) on 64 small pairs (`--foster`: also on the
10k x 8k pair, about 5 minutes).

The single pair does not shard across GPUs (the tree and the tracing are
global), so N > 1 runs N independent replicas, one per rank (torchrun), and
reports the max over ranks.

`--workload small_pairs_65536` measures the batched path instead: 65,536
independent small pairs (4-64 vertices), one step = their intersection areas
and area gradients on device-resident arrays, reported as pairs per second
(whole job; under torchrun each rank clips its own 65,536 pairs), next to
the plain per-pair GPU path (one sbc_clip_pair_device call per pair) and the
reference run pairwise on the host cores.

`--workload one_to_many_200k_10000` measures one 200,000-vertex jagged base
against 10,000 overlays (sizes log-uniform in [4, 5000], radii log-uniform in
[0.001R, 0.05R], centres uniform in the base's box), each overlay's result
being `seg base overlay` (sbc_clip_pairwise): one step = all 10,000 pairs on
device-resident inputs, reported as pairs per second, next to the plain
per-pair GPU path and the reference run pairwise on the host cores.

`--workload uneven_pairs_1m` measures 1,000,000 pairs with vertex counts
log-uniform in [3, 2048] per polygon plus 16 pairs of 200,000 vertices mixed
in: one step = every pair's intersection area and its gradient
(sbc_area_forward_device + sbc_area_backward_device), with the arenas cut
into chunks under the memory budget and each chunk's forward recomputed for
the backward pass.

`--impl reference` times the reference's own CPU (OpenMP) build
(oracle/_ref/seg, all host threads) on the same workload; when that build is
absent, the C restatement of the same algorithm (one thread).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "segment-tree-based-clipping_gb300"
for _p in (PKG, ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import sbclip_gen as gen  # noqa: E402

METRIC = "ms per 1M×1M clip"


def metric_of(workload: str) -> str:
    return {"pair_1m_1m": METRIC, "pair_200k_200k": "ms per 200k×200k clip",
            "pair_10k_8k": "ms per 10k×8k clip"}[workload]
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


JAGGED_DESC = ("jagged stars, R=%g, r=R(1+0.3g) clamped >= 0.2R, g = 8 octaves of value noise, "
               "base_freq=%d; overlay offset (0.25R, 0.1R), rotated 0.3 rad"
               % (gen.LARGE_R, gen.JAGGED_BASE_FREQ))


def workload(name: str):
    if name == "pair_1m_1m":
        b, c = gen.pair_large()
        desc = {"workload": "pair_1m_1m", "base_vertices": len(b), "overlay_vertices": len(c),
                "generator": JAGGED_DESC}
    elif name == "pair_200k_200k":
        b, c = gen.pair_large(n=200_000)
        desc = {"workload": "pair_200k_200k", "base_vertices": len(b), "overlay_vertices": len(c),
                "generator": JAGGED_DESC}
    elif name == "pair_10k_8k":
        b, c = gen.pair_small()
        desc = {"workload": "pair_10k_8k", "base_vertices": len(b), "overlay_vertices": len(c),
                "generator": "plain stars r=0.5+0.5u"}
    else:
        raise SystemExit(f"unknown workload {name}")
    return b, c, desc


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        os.unlink(self.path)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# What bounds each kernel that can dominate a step (ncu summaries in
# profiles/): "hbm" for byte-moving passes, "fp64" for the edge-pair
# classifier kernels (the FP64 pipe; GB300's FP64 rate is low), "latency" for
# dependent pointer chases and serial per-pair code, where neither HBM nor a
# pipe is busy.  The roofline entry reports the kernel against HBM bytes in
# every case and says which bound applies.
KERNEL_BOUND = {
    "k_os_scatter_u64": "hbm", "k_os_hist_u64": "hbm", "k_os_scatter_u32": "hbm",
    "k_os_hist_u32": "hbm", "k_scan_lb": "hbm", "k_setup_edges": "hbm", "k_edge_tree": "hbm",
    "k_alpha_classify": "hbm", "k_cover_count": "latency", "k_alpha_sort_long": "latency",
    "k_lr_jump_coop": "latency", "k_tr_jump_coop": "latency",
    "k_grid_scatter": "hbm", "k_edge_fbox": "hbm", "k_copy_runs": "hbm",
    "k_pair_exact": "fp64", "k_pw_cand_test": "fp64", "k_batch_cand": "fp64",
    "k_batch_cand_sweep": "fp64", "k_labels": "fp64", "k_batch_backward": "fp64",
    "k_grid_warp": "latency", "k_grid_small": "latency", "k_lr_jump": "latency",
    "k_tr_jump": "latency", "k_alpha_sort": "latency", "k_batch_back": "latency",
    "k_batch_front": "latency", "k_pw_pairs": "latency", "k_pw_pairs_lists": "latency",
    "k_pw_pairs_trace": "latency", "k_dedup": "latency", "k_batch_pw": "latency",
    "k_batch_pw2": "latency", "k_batch_labels": "fp64", "k_batch_back2": "latency",
    "k_comp_succ": "hbm",
}

# Pipe and issue utilisation of kernels that HBM does not bound, from one ncu
# capture each (percentages, so a capture of a smaller case of the same
# kernel applies), keyed (kernel, workload).
_BATCH_NCU = "profiles/k_batch_small_pairs_8192.md (8,192 pairs, the same kernel)"
PIPES = {
    ("k_batch_pw2", "small_pairs_65536"): {
        "fp64_pipe_pct_active": 11.0, "warps_active_pct": 27.1, "issue_active_pct": 28.3,
        "stall_cycles_per_issue": {"long_scoreboard": 7.0, "no_instruction": 3.3, "wait": 2.9},
        "source": _BATCH_NCU},
    ("k_batch_pw", "small_pairs_65536"): {
        "fp64_pipe_pct_active": 27.4, "warps_active_pct": 29.0, "issue_active_pct": 29.2,
        "stall_cycles_per_issue": {"long_scoreboard": 5.8, "no_instruction": 3.9, "wait": 3.5},
        "source": _BATCH_NCU},
    ("k_batch_front", "small_pairs_65536"): {
        "fp64_pipe_pct_active": 18.4, "warps_active_pct": 32.4, "issue_active_pct": 44.4,
        "source": _BATCH_NCU},
    ("k_batch_backward", "small_pairs_65536"): {
        "fp64_pipe_pct_active": 75.2, "warps_active_pct": 22.7, "issue_active_pct": 14.6,
        "source": _BATCH_NCU},
}

# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
# kernels captured with ncu on the named workload, keyed (kernel, workload).
# A capture on a smaller case of the same kernel is scaled by the units it
# processed where the traffic grows in proportion (said in the source note).
TRAFFIC = {
    # a radix pass moves 16 algorithmic bytes per key; the capture is a pass
    # of the 2M vertex keys (32 MB algorithmic), scaled to the average launch
    ("k_os_scatter_u32", "pair_1m_1m"): {
        "per_algorithmic_byte": (17076480 + 5888) / 32.0e6,
        "source": "profiles/k_os_scatter_u32_pair_1m_1m.md (one pass of 2M 32-bit vertex keys: "
                  "the 16 MB input from DRAM, the output left in L2 for the next pass; scaled "
                  "to the launch's keys)"},
    ("k_pair_exact", "pair_1m_1m"): {
        "bytes": 163223808 + 11570432, "source": "profiles/k_pair_exact_pair_1m_1m.md"},
}


def roofline_of(prof_b: dict, workload_name: str, fallback_bytes=None):
    """Roofline entry of the kernel with the largest device time in a
    per-launch profile {name: (ms, launches, stated bytes)}."""
    if not prof_b:
        return None
    pk, kind = peaks()
    name, (tot_ms, n_l, by) = max(prof_b.items(), key=lambda kv: kv[1][0])
    per_ms = tot_ms / max(n_l, 1)
    ab = by / max(n_l, 1) if by else (fallback_bytes(name, n_l) if fallback_bytes else None)
    achieved = ab / (per_ms * 1e-3) / 1e9 if ab else None
    tr = TRAFFIC.get((name, workload_name))
    traffic = None
    if tr and "bytes" in tr:
        traffic = tr["bytes"]
    elif tr and ab:
        traffic = tr["per_algorithmic_byte"] * ab
    bound = KERNEL_BOUND.get(name, "hbm")
    pipes = PIPES.get((name, workload_name))
    return {"kernel": name, "bound": bound, "achieved": achieved,
            "pipes": pipes if bound != "hbm" else None,
            "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"] if achieved else None,
            "traffic": traffic,
            "traffic_source": tr["source"] if tr else None,
            "algorithmic_bytes_per_launch": ab, "ms_per_launch": per_ms,
            "share_of_step": tot_ms / max(sum(v[0] for v in prof_b.values()), 1e-9),
            "peak_source": kind}


# Algorithmic bytes per launch of the kernels that can dominate a step, from
# the run's statistics.  The exact candidate kernel counts 64 B per
# box-overlapping edge pair (the two edges' coordinates); the tree kernels
# count their inputs and outputs once.
def algorithmic_bytes(kernel: str, st: dict, launches: int):
    E = st["edges"]
    per = max(launches, 1)
    if kernel == "k_pair_exact":
        # the two edges' coordinates of every box-overlapping pair (64 B)
        return 64.0 * st["grid_pairs"] / per
    if kernel == "k_find_leaves":
        return 16.0 * E + 8.0 * E
    if kernel == "k_edge_range":
        return 16.0 * E + 8.0 * E
    return None


def run_gb300(args, rank: int, world: int):
    import torch
    import sbclip

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    b, c, desc = workload(args.workload)
    nb, nc = len(b), len(c)
    d_b = torch.from_numpy(np.ascontiguousarray(b)).to(f"cuda:{dev}")
    d_c = torch.from_numpy(np.ascontiguousarray(c)).to(f"cuda:{dev}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    clip = sbclip.Clipper(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    for _ in range(args.warmup):
        clip.clip_pair_device(d_b.data_ptr(), nb, d_c.data_ptr(), nc, sp)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    st_launch = sbclip.kernel_launches()
    times = []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            clip.clip_pair_device(d_b.data_ptr(), nb, d_c.data_ptr(), nc, sp)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    launches = sbclip.kernel_launches() - st_launch
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    ms = float(np.mean(times))
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    stats = clip.stats()

    # ---- per-kernel device times: one more step, outside the timed region,
    # with every launch bracketed by CUDA events on the library's stream
    flush.fill_(1.0)
    torch.cuda.synchronize()
    sbclip.profile_begin()
    clip.clip_pair_device(d_b.data_ptr(), nb, d_c.data_ptr(), nc, sp)
    torch.cuda.synchronize()
    prof_b = sbclip.profile_end(with_bytes=True)
    prof = {k: (v[0], v[1]) for k, v in prof_b.items()}
    if args.timeline and rank == 0:
        write_timeline(args.timeline, sbclip.profile_timeline())

    # ---- end to end through the host C ABI (sbc_clip_pair): host buffers in,
    # host->device and device->host copies inside every step
    e2e_times = []
    off = xy = None
    # untimed warm-up of the host path (its first call sizes the context's
    # input staging and pinned result memory)
    for _ in range(args.warmup):
        clip.clip_pair_flat(b, c, copy=False)
    for i in range(max(args.steps, 1)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        off, xy = clip.clip_pair_flat(b, c, copy=False)
        e2e_times.append((time.perf_counter() - t0) * 1e3)
    nrings = len(off) - 1
    nverts = int(xy.shape[0])
    e2e = {"value": float(np.mean(e2e_times)), "unit": "ms",
           "h2d_bytes_per_step": int(16 * (nb + nc)),
           "d2h_bytes_per_step": int(4 * (nrings + 1) + 16 * nverts)}

    # ---- roofline of the dominant kernel (the bytes the launch sites state,
    # else the table above)
    roof = roofline_of(prof_b, args.workload, lambda k, n: algorithmic_bytes(k, stats, n))
    top = sorted(prof.items(), key=lambda kv: -kv[1][0])[:10]

    out = {
        "metric": metric_of(args.workload),
        "value": ms, "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded star polygons)",
        "config": dict(desc, parallelism="replicas" if world > 1 else "single",
                       l2="flushed between steps (256 MiB write)"),
        "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
        "kernels_top": {k: {"ms_per_step": v[0], "launches_per_step": v[1]} for k, v in top},
        # the profiled step's launches, each bracketed by CUDA events: their
        # summed time next to the device time per step shows the gaps between
        # kernels (host round trips, launch latency)
        "kernel_ms_per_step": float(sum(v[0] for v in prof.values())),
        "launches_per_step": int(sum(v[1] for v in prof.values())),
        "stats": stats, "clocks": clk.summary(),
        "counts": {"rings": nrings, "vertices": nverts, "unique_intersections": stats["unique"],
                   "candidates_tested_per_s": stats["candidates_tested"] / (ms * 1e-3)},
    }
    clip.close()
    if args.workload == "pair_1m_1m" and not args.no_batched:
        out["batched"] = batched_summary(args, rank, world)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(b, c, args)
        out["cpu_baseline"]["others"] = extra_cpu_baselines(args.foster)
    return out


def cpu_baseline(b, c, args, steps: int = 1):
    """The reference's CPU build (all host threads) on the full workload."""
    import oracle_py as O
    threads = os.cpu_count() or 1
    if O.ref_available():
        vals = []
        for _ in range(steps):
            t0 = time.perf_counter()
            res = O.run_reference(b, [c], threads=threads, precision=6, timeout=1800)
            wall = (time.perf_counter() - t0) * 1e3
            tl = res["time_line"]
            vals.append(tl[-1] / 1e3 if tl else wall)
        return {"value": float(np.mean(vals)), "unit": "ms", "cores": threads, "kind": "reference",
                "sample": f"{steps} full {args.workload} clip(s), reference TIME-line total "
                          f"(OMP_NUM_THREADS={threads})"}
    vals = []
    for _ in range(steps):
        t0 = time.perf_counter()
        O.clip(b, [c])
        vals.append((time.perf_counter() - t0) * 1e3)
    return {"value": float(np.mean(vals)), "unit": "ms", "cores": 1, "kind": "port",
            "sample": f"{steps} full {args.workload} clip(s) by the C restatement (1 thread)"}


# ---------------------------------------------------------------- small-pair batches
SMALL_PAIRS = 65536


def small_pairs_workload(n: int, seed: int):
    pairs = gen.small_pairs(n, seed=seed)
    desc = {"workload": f"small_pairs_{n}", "pairs": n, "vertices_per_polygon": "U[4,64]",
            "generator": "plain stars r=0.5+0.5u, overlay centre offset U[-0.5,0.5]^2"}
    return pairs, desc


def reference_pairs_per_s(pairs, threads: int):
    """The reference's CPU build run pairwise (one process per pair, `threads`
    processes at a time) on a sample of pairs: clipped pairs per second."""
    import oracle_py as O
    from concurrent.futures import ThreadPoolExecutor
    if not O.ref_available():
        t0 = time.perf_counter()
        for b, c in pairs:
            O.clip(b, [c])
        return len(pairs) / (time.perf_counter() - t0), 1, "port"
    def one(bc):
        try:  # the reference crashes on some inputs (reads past its arrays)
            O.run_reference(bc[0], [bc[1]], threads=1, precision=6, timeout=60)
            return 1
        except RuntimeError:
            return 0

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, pairs))
    return len(pairs) / (time.perf_counter() - t0), threads, "reference"


def max_over_ranks(x: float, world: int, device: str) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_job(nb, nc, rank: int, world: int, hits=None):
    """This rank's pairs of one job partitioned over the ranks by estimated
    cost (longest processing time first), and a summary of the partition."""
    import shard
    costs = shard.pair_costs(nb, nc, hits)
    parts = shard.lpt_partition(costs, world)
    return parts[rank], shard.shard_summary(costs, parts)


def gather_check(local: dict, n_total: int, args):
    """Host-side gather of per-pair outputs on rank 0 (outside the timed
    region); returns the number of pairs gathered (rank 0) or None."""
    import shard
    got = shard.gather_outputs(local, n_total, group=getattr(args, "gloo", None))
    return None if got is None else len(got)


def run_small_pairs(args, rank: int, world: int):
    """One step = intersection areas of every pair (sbc_area_forward_device)
    and their gradient (sbc_area_backward_device, reusing the forward's
    records), all pairs in one launch each; inputs resident on the device."""
    import torch
    import sbclip

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    n = args.pairs or SMALL_PAIRS
    n_total = n * world  # weak scaling: n pairs per GPU in one job
    pairs, desc = small_pairs_workload(n_total, 4000)
    shard_info = None
    mine = np.arange(n_total)
    if world > 1:
        mine, shard_info = shard_job([len(b) for b, _ in pairs], [len(c) for _, c in pairs],
                                     rank, world)
        pairs = [pairs[i] for i in mine]
        n = len(pairs)
    bases, ovs = [b for b, _ in pairs], [c for _, c in pairs]
    bxy, boff = sbclip.pack_polygons(bases)
    cxy, coff = sbclip.pack_polygons(ovs)
    cuda = f"cuda:{dev}"
    t = {k: torch.from_numpy(v).to(cuda) for k, v in
         (("bxy", bxy), ("boff", boff), ("cxy", cxy), ("coff", coff))}
    area = torch.zeros(n, dtype=torch.float64, device=cuda)
    st = torch.zeros(n, dtype=torch.int32, device=cuda)
    ga = torch.ones(n, dtype=torch.float64, device=cuda)
    gb = torch.zeros_like(t["bxy"])
    gc = torch.zeros_like(t["cxy"])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=cuda)
    clip = sbclip.Clipper(dev)
    # an explicit stream: the graph runs, and the events time it, on one stream
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    a = (n, t["bxy"].data_ptr(), t["boff"].data_ptr(), t["cxy"].data_ptr(), t["coff"].data_ptr())

    # the autotuner picks the batch engine's block sizes (and the small/large
    # split where it applies) by timing forward + backward on this batch,
    # outside the timed region; results do not depend on them
    tuned = clip.autotune_batch_device(*a, ga.data_ptr(), gb.data_ptr(), gc.data_ptr(), sp)
    # the whole forward + backward step as one CUDA graph, recorded once
    graph = clip.area_graph(*a, ga.data_ptr(), gb.data_ptr(), gc.data_ptr(), area.data_ptr(),
                            st.data_ptr(), sp)

    def step():
        graph.launch(sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    l0 = sbclip.kernel_launches()
    times = []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    launches = sbclip.kernel_launches() - l0
    ms = float(np.mean(times))
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms], device=cuda)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    n_ok = int((st == 0).sum().item())
    # per-kernel times of one more step, run as the separate calls the graph
    # was recorded from (a graph replay has no per-launch events)
    torch.cuda.synchronize()
    sbclip.profile_begin()
    clip.area_forward_device(*a, area.data_ptr(), st.data_ptr(), sp)
    clip.area_backward_device(*a, ga.data_ptr(), gb.data_ptr(), gc.data_ptr(), sp)
    torch.cuda.synchronize()
    prof_b = sbclip.profile_end(with_bytes=True)
    graph.close()
    prof = {k: (v[0], v[1]) for k, v in prof_b.items()}
    # end to end through the host-array C ABI (sbc_area_forward and
    # sbc_area_backward on the packed host arrays): inputs copied in, areas
    # and gradients copied out (the host backward call runs its own forward)
    e2e_t = []
    ones = np.ones(n)
    for _ in range(args.warmup):
        clip.area_forward_packed(bxy, boff, cxy, coff)
        clip.area_backward_packed(bxy, boff, cxy, coff, ones)
    for _ in range(max(args.steps, 1)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        clip.area_forward_packed(bxy, boff, cxy, coff)
        clip.area_backward_packed(bxy, boff, cxy, coff, ones)
        e2e_t.append((time.perf_counter() - t0) * 1e3)
    in_bytes = 16 * (int(boff[-1]) + int(coff[-1])) + 16 * (n + 1)
    gathered = gather_check({int(i): float(a) for i, a in zip(mine, area.cpu().numpy())},
                            n_total, args) if world > 1 else n_total
    e2e_ms = max_over_ranks(float(np.mean(e2e_t)), world, cuda)
    e2e = {"value": n_total / (e2e_ms * 1e-3), "unit": "pairs/s",
           "h2d_bytes_per_step": 2 * in_bytes + 8 * n,
           "d2h_bytes_per_step": 12 * n + 16 * (int(boff[-1]) + int(coff[-1]))}
    # the plain per-pair GPU path (one sbc_clip_pair_device call per pair, forward only)
    sample = 256
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p in range(sample):
        clip.clip_pair_device(t["bxy"].data_ptr() + 16 * int(boff[p]), int(boff[p + 1] - boff[p]),
                              t["cxy"].data_ptr() + 16 * int(coff[p]), int(coff[p + 1] - coff[p]), sp)
    torch.cuda.synchronize()
    per_pair = sample / (time.perf_counter() - t0)
    roof = roofline_of(prof_b, desc["workload"])
    out = {
        "metric": "clipped pairs/s, batched area forward+backward, 65,536 small pairs",
        "value": n_total / (ms * 1e-3), "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded star polygons)",
        "config": dict(desc, parallelism=("one job sharded by cost (LPT), gathered on rank 0"
                                          if world > 1 else "single"),
                       shard=shard_info, gathered_pairs=gathered,
                       l2="flushed between steps (256 MiB write)",
                       launch="one CUDA graph per step (area forward + backward)",
                       autotuned={k: v for k, v in tuned.items() if k != "best_ms"}),
        "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
        "kernels_top": {k: {"ms_per_step": v[0], "launches_per_step": v[1]}
                        for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])[:6]},
        "clocks": clk.summary(),
        "counts": {"pairs_ok": n_ok, "per_pair_gpu_path_pairs_per_s": per_pair,
                   "per_pair_sample": sample,
                   "batched_over_per_pair": (n_total / (ms * 1e-3)) / per_pair},
    }
    if rank == 0 and not args.no_cpu_baseline:
        v, cores, kind2 = reference_pairs_per_s(pairs[:256], os.cpu_count() or 1)
        out["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": cores, "kind": kind2,
                               "sample": "256 pairs clipped pairwise (forward only; the "
                                         "reference computes no gradients)"}
    clip.close()
    return out


ONE_TO_MANY = (200_000, 10_000)
ONE_TO_MANY_METRIC = "clipped pairs/s, one 200k-vertex base x 10,000 overlays, pairwise forward"


def one_to_many_workload(n_overlays: int | None = None, per_gpu: int = 1):
    nb, nov = ONE_TO_MANY
    nov *= per_gpu
    base, ovs = gen.one_to_many(n_base=nb, n_overlays=nov, seed=3000)
    if n_overlays is not None:
        ovs = ovs[:n_overlays]
        nov = len(ovs)
    desc = {"workload": f"one_to_many_{nb // 1000}k_{nov}", "base_vertices": nb,
            "overlays": nov, "overlay_vertices": int(sum(len(o) for o in ovs)),
            "generator": "jagged base R=1000; plain-star overlays, sizes log-U[4,5000], radii "
                         "log-U[0.001R,0.05R], centres U(base box)"}
    return base, ovs, desc


def run_one_to_many(args, rank: int, world: int):
    """One step = every overlay's pairwise result (sbc_clip_pairwise_device)
    on device-resident inputs."""
    import torch
    import sbclip

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    # weak scaling: 10,000 overlays per GPU in one job against the replicated base
    base, ovs, desc = one_to_many_workload(args.overlays, per_gpu=world)
    nov_total = len(ovs)
    cuda = f"cuda:{dev}"
    shard_info = None
    mine = np.arange(nov_total)
    if world > 1:
        # cost: n log n plus K estimated per size class from a sampled run
        # (every 25th overlay; the same sample and result on every rank)
        sample = np.arange(0, nov_total, 25)
        sxy, soff = sbclip.pack_polygons([ovs[i] for i in sample])
        pre = sbclip.Clipper(dev)
        pr, ro, _xy, _st = pre.clip_pairwise_flat(base, sxy, soff, copy=True)
        pre.close()
        k_sample = np.array([ro[pr[i + 1]] - ro[pr[i]] for i in range(len(sample))], np.float64)
        import shard
        nc_all = np.array([len(o) for o in ovs])
        hits = shard.estimate_hits(len(base) + nc_all, sample, k_sample)
        mine, shard_info = shard_job(np.full(nov_total, len(base)), nc_all, rank, world, hits)
        ovs = [ovs[i] for i in mine]
    nov = len(ovs)
    cxy, coff = sbclip.pack_polygons(ovs)
    tb = torch.from_numpy(np.ascontiguousarray(base)).to(cuda)
    tc = torch.from_numpy(cxy).to(cuda)
    to = torch.from_numpy(coff).to(cuda)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=cuda)
    clip = sbclip.Clipper(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def step():
        return clip.clip_pairwise_device(tb.data_ptr(), len(base), nov, tc.data_ptr(),
                                         to.data_ptr(), sp)

    if args.job_only:
        # profiling mode: the job alone, default settings, no JSON line
        for _ in range(args.job_only):
            nr, nv = step()
        torch.cuda.synchronize()
        print(f"job ok: {nov} overlays, {nr} rings, {nv} vertices, {clip.pairwise_info()}",
              file=sys.stderr)
        clip.close()
        return None

    # the autotuner picks the big-pair split and the grid cell width (outside
    # the timed region; results do not depend on them)
    tuned = clip.autotune_pairwise_device(tb.data_ptr(), len(base), nov, tc.data_ptr(),
                                          to.data_ptr(), sp)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    l0 = sbclip.kernel_launches()
    times = []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            nr, nv = step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    launches = sbclip.kernel_launches() - l0
    info = clip.pairwise_info()
    ms = float(np.mean(times))
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms], device=cuda)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    # per-kernel times of one more step with the big overlays on one worker:
    # kernels on concurrent worker streams would each be timed with the
    # others' work inside their event pairs
    torch.cuda.synchronize()
    workers = clip.pairwise_workers()
    clip.set_pairwise_workers(1)
    sbclip.profile_begin()
    step()
    torch.cuda.synchronize()
    prof_b = sbclip.profile_end(with_bytes=True)
    clip.set_pairwise_workers(workers)
    prof = {k: (v[0], v[1]) for k, v in prof_b.items()}
    # end to end through the host-array C ABI (sbc_clip_pairwise): inputs
    # copied in and every ring copied out, inside each step
    e2e_t = []
    d2h = 0
    for _ in range(args.warmup):
        clip.clip_pairwise_flat(base, cxy, coff, sp, copy=False)
    for _ in range(max(args.steps, 1)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pr, ro, xy, stt = clip.clip_pairwise_flat(base, cxy, coff, sp, copy=False)
        e2e_t.append((time.perf_counter() - t0) * 1e3)
        d2h = ro.nbytes + xy.nbytes
        n_ok = int((stt == 0).sum())
    e2e_ms = max_over_ranks(float(np.mean(e2e_t)), world, cuda)
    e2e = {"value": nov_total / (e2e_ms * 1e-3), "unit": "pairs/s",
           "h2d_bytes_per_step": int(base.nbytes + cxy.nbytes + coff.nbytes),
           "d2h_bytes_per_step": int(d2h)}
    gathered = nov_total
    if world > 1:
        counts = np.diff(pr)
        gathered = gather_check({int(i): int(counts[j]) for j, i in enumerate(mine)},
                                nov_total, args)
    # area forward + backward of every pair (the gradient of the shared base
    # summed over the overlays): a separate figure next to the forward metric
    fb_area = torch.zeros(nov, dtype=torch.float64, device=cuda)
    fb_g = torch.ones(nov, dtype=torch.float64, device=cuda)
    fb_gb = torch.zeros_like(tb)
    fb_gc = torch.zeros_like(tc)
    fb_t = []
    for k in range(args.warmup + max(args.steps, 1)):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        clip.pairwise_area_device(tb.data_ptr(), len(base), nov, tc.data_ptr(), to.data_ptr(),
                                  fb_area.data_ptr(), None, sp)
        clip.pairwise_area_backward_device(tb.data_ptr(), len(base), nov, tc.data_ptr(),
                                           to.data_ptr(), fb_g.data_ptr(), fb_gb.data_ptr(),
                                           fb_gc.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            fb_t.append(e0.elapsed_time(e1))
    # the plain per-pair GPU path: one sbc_clip_pair_device call per overlay
    sample = 64
    rng = np.random.default_rng(5)
    pick = rng.choice(nov, sample, replace=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p in pick:
        clip.clip_pair_device(tb.data_ptr(), len(base), tc.data_ptr() + 16 * int(coff[p]),
                              int(coff[p + 1] - coff[p]), sp)
    torch.cuda.synchronize()
    per_pair = sample / (time.perf_counter() - t0)
    roof = roofline_of(prof_b, desc["workload"])
    value = nov_total / (ms * 1e-3)
    fb_ms = max_over_ranks(float(np.mean(fb_t)), world, cuda)
    out = {
        "metric": ONE_TO_MANY_METRIC,
        "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded star polygons)",
        "config": dict(desc, parallelism=("one job sharded by cost (LPT), base replicated, "
                                          "gathered on rank 0" if world > 1 else "single"),
                       shard=shard_info, gathered_pairs=gathered,
                       l2="flushed between steps (256 MiB write)",
                       autotuned={"big_pair_split_records": tuned["split"],
                                  "grid_cell_factor": tuned["cell_factor"]}),
        "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
        "kernels_top": {k: {"ms_per_step": v[0], "launches_per_step": v[1]}
                        for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])[:8]},
        "clocks": clk.summary(),
        "counts": {"pairs_ok": n_ok, "rings": nr, "ring_vertices": nv,
                   "pairs_by_pair_pipeline": info["fallback_pairs"],
                   "pairs_by_pipeline_rows_a10_a18": info["big_pairs"],
                   "unique_intersections": info["unique"],
                   "box_overlapping_edge_pairs_tested": info["tested"],
                   "edge_pairs_tested_per_s": info["tested"] / (ms * 1e-3),
                   "per_pair_gpu_path_pairs_per_s": per_pair, "per_pair_sample": sample,
                   "batched_over_per_pair": value / per_pair,
                   "area_forward_backward_ms": fb_ms,
                   "area_forward_backward_pairs_per_s": nov_total / (fb_ms * 1e-3)},
    }
    if rank == 0 and not args.no_cpu_baseline:
        sample_cpu = [(base, ovs[int(p)]) for p in pick[:32]]
        v, cores, kind2 = reference_pairs_per_s(sample_cpu, os.cpu_count() or 1)
        out["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": cores, "kind": kind2,
                               "sample": "32 of the overlays, each clipped against the base by "
                                         "its own reference run"}
    clip.close()
    return out


UNEVEN = (1_000_000, 16)
UNEVEN_METRIC = ("clipped pairs/s, area forward+backward, 1M uneven pairs (3-2048 vertices) "
                 "+ 16 pairs of 200k")


def uneven_workload():
    n, nl = UNEVEN
    bxy, boff, cxy, coff = gen.uneven_pairs(n, nl, seed=5000)
    desc = {"workload": "uneven_pairs_1m", "pairs": n + nl, "large_pairs": nl,
            "vertices": int(boff[-1] + coff[-1]),
            "generator": "plain stars, sizes log-U[3,2048], stratified angles, overlay centre "
                         "U[-0.5,0.5]^2; 16 jagged 200k-vertex pairs (R=1000) mixed in"}
    return bxy, boff, cxy, coff, desc


def run_uneven(args, rank: int, world: int):
    """One step = areas and area gradients of every pair on device arrays."""
    import torch
    import sbclip

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    bxy, boff, cxy, coff, desc = uneven_workload()
    n = len(boff) - 1
    cuda = f"cuda:{dev}"
    t = {k: torch.from_numpy(v).to(cuda) for k, v in
         (("bxy", bxy), ("boff", boff), ("cxy", cxy), ("coff", coff))}
    area = torch.zeros(n, dtype=torch.float64, device=cuda)
    st = torch.zeros(n, dtype=torch.int32, device=cuda)
    ga = torch.ones(n, dtype=torch.float64, device=cuda)
    gb = torch.zeros_like(t["bxy"])
    gc = torch.zeros_like(t["cxy"])
    clip = sbclip.Clipper(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    a = (n, t["bxy"].data_ptr(), t["boff"].data_ptr(), t["cxy"].data_ptr(), t["coff"].data_ptr())

    def step():
        clip.area_forward_device(*a, area.data_ptr(), st.data_ptr(), sp)
        clip.area_backward_device(*a, ga.data_ptr(), gb.data_ptr(), gc.data_ptr(), sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    l0 = sbclip.kernel_launches()
    times = []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    launches = sbclip.kernel_launches() - l0
    binfo = clip.batch_info()
    ms = float(np.mean(times))
    n_ok = int((st == 0).sum().item())
    torch.cuda.synchronize()
    sbclip.profile_begin()
    step()
    torch.cuda.synchronize()
    prof_b = sbclip.profile_end(with_bytes=True)
    prof = {k: (v[0], v[1]) for k, v in prof_b.items()}
    # end to end through the host-array C ABI (the host backward runs its own forward)
    t0 = time.perf_counter()
    clip.area_forward_packed(bxy, boff, cxy, coff)
    clip.area_backward_packed(bxy, boff, cxy, coff, np.ones(n))
    e2e_ms = (time.perf_counter() - t0) * 1e3
    in_bytes = bxy.nbytes + cxy.nbytes + boff.nbytes + coff.nbytes
    e2e = {"value": n / (e2e_ms * 1e-3), "unit": "pairs/s",
           "h2d_bytes_per_step": 2 * in_bytes + 8 * n,
           "d2h_bytes_per_step": 12 * n + bxy.nbytes + cxy.nbytes, "steps": 1}
    # the plain per-pair GPU path on a sample of the pairs
    rng = np.random.default_rng(7)
    pick = rng.choice(n, 128, replace=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p in pick:
        clip.clip_pair_device(t["bxy"].data_ptr() + 16 * int(boff[p]), int(boff[p + 1] - boff[p]),
                              t["cxy"].data_ptr() + 16 * int(coff[p]), int(coff[p + 1] - coff[p]),
                              sp)
    torch.cuda.synchronize()
    per_pair = len(pick) / (time.perf_counter() - t0)
    roof = roofline_of(prof_b, desc["workload"])
    value = n / (ms * 1e-3)
    out = {
        "metric": UNEVEN_METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded star polygons)",
        "config": dict(desc, parallelism="single", l2="inputs (10 GB) larger than L2",
                       arena_chunks=binfo["chunks"]),
        "e2e": e2e, "gpu_launches": int(launches), "roofline": roof,
        "kernels_top": {k: {"ms_per_step": v[0], "launches_per_step": v[1]}
                        for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])[:8]},
        "clocks": clk.summary(),
        "counts": {"pairs_ok": n_ok, "large_pairs": binfo["large_pairs"],
                   "per_pair_gpu_path_pairs_per_s": per_pair, "per_pair_sample": len(pick),
                   "batched_over_per_pair": value / per_pair},
    }
    if rank == 0 and not args.no_cpu_baseline:
        sample = [(bxy[boff[p]:boff[p + 1]], cxy[coff[p]:coff[p + 1]]) for p in pick[:64]]
        v, cores, kind2 = reference_pairs_per_s(sample, os.cpu_count() or 1)
        out["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": cores, "kind": kind2,
                               "sample": "64 random pairs clipped pairwise (forward only)"}
    clip.close()
    return out


def batched_summary(args, rank: int, world: int):
    """The batched half of the headline metric, measured in the same run: the
    small-pair batch (area forward + backward, one CUDA graph launch per step)
    and one base against many overlays (forward, and area forward + backward),
    each next to the plain per-pair GPU path (one sbc_clip_pair_device call
    per pair) on the same inputs."""
    sub = argparse.Namespace(**vars(args))
    sub.pairs = None
    sub.overlays = None
    sub.job_only = 0
    sp = run_small_pairs(sub, rank, world)
    om = run_one_to_many(sub, rank, world)
    c3 = om["counts"]
    out = {
        "target": "batched forward+backward pairs/s >= 5x the plain per-pair GPU path",
        "small_pairs_65536": {
            "metric": sp["metric"], "pairs_per_s": sp["value"], "ms_per_step": sp["ms_per_step"],
            "launch": "one CUDA graph per step (area forward + backward)",
            "autotuned": sp["config"]["autotuned"],
            "e2e_pairs_per_s": sp["e2e"]["value"],
            "per_pair_gpu_path_pairs_per_s": sp["counts"]["per_pair_gpu_path_pairs_per_s"],
            "forward_backward_over_per_pair": sp["counts"]["batched_over_per_pair"],
            "gpu_launches": sp["gpu_launches"], "roofline": sp["roofline"],
            "kernels_top": dict(list(sp["kernels_top"].items())[:4]), "clocks": sp["clocks"],
            "cpu_baseline": sp.get("cpu_baseline")},
        "one_to_many_200k_10000": {
            "metric": "clipped pairs/s, one 200k-vertex base x 10,000 overlays",
            "forward_pairs_per_s": om["value"], "forward_ms_per_step": om["ms_per_step"],
            "forward_backward_pairs_per_s": c3["area_forward_backward_pairs_per_s"],
            "forward_backward_ms_per_step": c3["area_forward_backward_ms"],
            "e2e_forward_pairs_per_s": om["e2e"]["value"],
            "per_pair_gpu_path_pairs_per_s": c3["per_pair_gpu_path_pairs_per_s"],
            "forward_over_per_pair": c3["batched_over_per_pair"],
            "forward_backward_over_per_pair":
                c3["area_forward_backward_pairs_per_s"] / c3["per_pair_gpu_path_pairs_per_s"],
            "autotuned": om["config"]["autotuned"], "gpu_launches": om["gpu_launches"],
            "roofline": om["roofline"], "kernels_top": dict(list(om["kernels_top"].items())[:4]),
            "clocks": om["clocks"], "cpu_baseline": om.get("cpu_baseline")},
    }
    return out


def extra_cpu_baselines(foster_full: bool):
    """The reference's CPU build at one thread and at every host thread on the
    10k x 8k pair, and Foster's sequential code on 64 small pairs (and, with
    foster_full, on the 10k x 8k pair: about 5 minutes)."""
    import oracle_py as O
    out = []
    b, c = gen.pair_small()
    threads = os.cpu_count() or 1
    if O.ref_available():
        for t in (1, threads):
            t0 = time.perf_counter()
            res = O.run_reference(b, [c], threads=t, precision=6, timeout=600)
            wall = (time.perf_counter() - t0) * 1e3
            tl = res["time_line"]
            out.append({"impl": "reference", "cores": t, "workload": "pair_10k_8k",
                        "value": tl[-1] / 1e3 if tl else wall, "unit": "ms"})
    if O.foster_available():
        pairs = gen.small_pairs(64, seed=4000)
        t0 = time.perf_counter()
        for pb, pc in pairs:
            O.run_foster(pb, pc)
        out.append({"impl": "foster", "cores": 1, "workload": "small_pairs sample (64 pairs)",
                    "value": len(pairs) / (time.perf_counter() - t0), "unit": "pairs/s"})
        if foster_full:
            out.append({"impl": "foster", "cores": 1, "workload": "pair_10k_8k",
                        "value": O.run_foster(b, c)["ms"], "unit": "ms"})
    return out


def run_reference_arm(args):
    if args.workload.startswith("one_to_many"):
        base, ovs, desc = one_to_many_workload()
        steps = max(1, min(args.steps, 3))
        threads = os.cpu_count() or 1
        rng = np.random.default_rng(5)
        pick = rng.choice(len(ovs), 32 * steps, replace=False)
        vals = [reference_pairs_per_s([(base, ovs[int(p)]) for p in pick[32 * i:32 * (i + 1)]],
                                      threads) for i in range(steps)]
        v = float(np.mean([x[0] for x in vals]))
        cb = {"value": v, "unit": "pairs/s", "cores": vals[0][1], "kind": vals[0][2],
              "sample": f"{steps} x 32 overlays, each clipped against the base by its own run"}
        return {"impl": "reference", "metric": ONE_TO_MANY_METRIC, "value": v, "unit": "pairs/s",
                "n_gpus": args.gpus, "steps": steps, "warmup": 0, "ms_per_step": 32 / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded star polygons)",
                "config": dict(desc, parallelism="host cores"), "cpu_baseline": cb,
                "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
    if args.workload.startswith("small_pairs"):
        pairs, desc = small_pairs_workload(SMALL_PAIRS, 4000)
        steps = max(1, min(args.steps, 3))
        threads = os.cpu_count() or 1
        vals = [reference_pairs_per_s(pairs[256 * i:256 * (i + 1)], threads) for i in range(steps)]
        v = float(np.mean([x[0] for x in vals]))
        base = {"value": v, "unit": "pairs/s", "cores": vals[0][1], "kind": vals[0][2],
                "sample": f"{steps} x 256 pairs clipped pairwise (forward only)"}
        return {"impl": "reference",
                "metric": "clipped pairs/s, batched area forward+backward, 65,536 small pairs",
                "value": v, "unit": "pairs/s", "n_gpus": args.gpus, "steps": steps, "warmup": 0,
                "ms_per_step": 256 / v * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded star polygons)",
                "config": dict(desc, parallelism="host cores"), "cpu_baseline": base,
                "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
    b, c, desc = workload(args.workload)
    # each step is one full clip; the CPU arm is capped at 3 steps so the run
    # stays within a few minutes
    steps = max(1, min(args.steps, 3))
    base = cpu_baseline(b, c, args, steps=steps)
    out = {
        "impl": "reference",
        "metric": metric_of(args.workload),
        "value": base["value"], "unit": "ms", "n_gpus": args.gpus, "steps": steps,
        "warmup": 0, "ms_per_step": base["value"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded star polygons)",
        "config": dict(desc, parallelism="host cores"),
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return out


def write_timeline(path: str, tl) -> None:
    """One line per launch of the profiled step: start and duration (us), the
    stream, and the idle time on that stream since its previous launch ended
    (host round trips and launch latency)."""
    last_end: dict[int, float] = {}
    idle = {}
    with open(path, "w") as f:
        f.write("start_us  dur_us  stream  idle_us  kernel\n")
        for name, t0, dur, sid in tl:
            gap = (t0 - last_end[sid]) * 1e3 if sid in last_end else 0.0
            idle[sid] = idle.get(sid, 0.0) + max(gap, 0.0)
            last_end[sid] = t0 + dur
            f.write(f"{t0 * 1e3:9.1f} {dur * 1e3:7.1f} {sid:6d} {gap:8.1f}  {name}\n")
        end = max(last_end.values()) if last_end else 0.0
        f.write(f"# span {end * 1e3:.1f} us; idle per stream (us): "
                + ", ".join(f"{k}: {v:.1f}" for k, v in sorted(idle.items())) + "\n")


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="pair_1m_1m",
                    choices=["pair_1m_1m", "pair_200k_200k", "pair_10k_8k", "small_pairs_65536",
                             "one_to_many_200k_10000", "uneven_pairs_1m"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="pair_1m_1m only: leave out the batched measurements")
    ap.add_argument("--foster", action="store_true",
                    help="also time Foster's sequential code on the 10k x 8k pair (~5 min)")
    ap.add_argument("--job-only", type=int, default=0,
                    help="one_to_many only: run the job this many times and print no JSON "
                         "line (for profilers)")
    ap.add_argument("--timeline", default=None,
                    help="pair workloads: write the profiled step's launches (start, duration, "
                         "stream, idle gap before each) to this file")
    ap.add_argument("--pairs", type=int, default=None,
                    help="small_pairs only: number of pairs (default 65,536)")
    ap.add_argument("--overlays", type=int, default=None,
                    help="one_to_many only: use the first N overlays of the workload")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference_arm(args)), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        # host-side gathers of per-pair outputs (no device collective on the data path)
        args.gloo = dist.new_group(backend="gloo")
    if args.workload.startswith("small_pairs"):
        out = run_small_pairs(args, rank, world)
    elif args.workload.startswith("one_to_many"):
        out = run_one_to_many(args, rank, world)
    elif args.workload.startswith("uneven"):
        out = run_uneven(args, rank, world)
    else:
        out = run_gb300(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
