"""GPU parity of the one-base-many-overlays call (sbc_clip_pairwise).

Every overlay's rings must equal sbc_clip_pair(base, overlay) bit for bit:
the pair pipeline is itself pinned to the reference's CPU build, and
`seg base overlay` run once per overlay is what the reference offers for this
workload.  The cases cover overlays inside, outside and across the base's
boundary, inputs that leave the batched path's conditions (a shared x value, a
vertical edge, a polygon the size of the base), an overlay that contains the
whole base, and too-short overlays.
"""
from __future__ import annotations

import numpy as np
import pytest

import sbclip_gen as gen
from conftest import rings_equal

pytestmark = pytest.mark.gpu


def _check(clipper, base, overlays):
    got, st = clipper.clip_pairwise(base, overlays)
    assert len(got) == len(overlays)
    bad = []
    for i, c in enumerate(overlays):
        if len(c) < 3:
            assert st[i] == 1, i
            assert got[i] == []
            continue
        want = clipper.clip_pair(base, c)
        assert st[i] == 0, (i, st[i])
        if not rings_equal(got[i], want):
            bad.append(i)
    assert not bad, f"{len(bad)} overlays differ, first {bad[:8]}"
    return got


def test_pairwise_random_overlays(clipper):
    base, ovs = gen.one_to_many(n_base=20_000, n_overlays=300, seed=3100, hi=2000,
                                near_boundary=0.5)
    got = _check(clipper, base, ovs)
    info = clipper.pairwise_info()
    assert info["fallback_pairs"] <= len(ovs) // 20, info
    assert info["unique"] > 100, info
    assert sum(len(r) for r in got) > 50


def test_pairwise_cell_factor_does_not_change_results(clipper):
    base, ovs = gen.one_to_many(n_base=5_000, n_overlays=120, seed=3200, hi=800,
                                near_boundary=0.6)
    ref, _ = clipper.clip_pairwise(base, ovs)
    for f in (0.25, 4.0):
        clipper.set_pairwise_cell_factor(f)
        try:
            got, _ = clipper.clip_pairwise(base, ovs)
        finally:
            clipper.set_pairwise_cell_factor(1.0)
        assert all(rings_equal(a, b) for a, b in zip(got, ref))


def test_pairwise_split_does_not_change_results(clipper):
    """Every overlay with at least one record through the data-parallel rows
    A9-A18, then none: the same rings as the default split."""
    base, ovs = gen.one_to_many(n_base=8_000, n_overlays=150, seed=3250, hi=1500,
                                near_boundary=0.7)
    ref, _ = clipper.clip_pairwise(base, ovs)
    try:
        for split in (1, 1 << 30):
            clipper.set_pairwise_split(split)
            got, st = clipper.clip_pairwise(base, ovs)
            assert (st == 0).all()
            info = clipper.pairwise_info()
            if split == 1:
                assert info["big_pairs"] > 50, info
            else:
                assert info["big_pairs"] == 0, info
            assert all(rings_equal(a, b) for a, b in zip(got, ref))
    finally:
        clipper.set_pairwise_split(8192)
    for i in range(0, len(ovs), 10):
        assert rings_equal(ref[i], clipper.clip_pair(base, ovs[i])), i


def test_pairwise_autotune(clipper):
    torch = pytest.importorskip("torch")
    import sbclip
    base, ovs = gen.one_to_many(n_base=6_000, n_overlays=100, seed=3260, hi=1200,
                                near_boundary=0.6)
    ref, _ = clipper.clip_pairwise(base, ovs)
    cxy, coff = sbclip.pack_polygons(ovs)
    tb = torch.from_numpy(np.ascontiguousarray(base)).to("cuda:0")
    tc = torch.from_numpy(cxy).to("cuda:0")
    to = torch.from_numpy(coff).to("cuda:0")
    try:
        t = clipper.autotune_pairwise_device(tb.data_ptr(), len(base), len(ovs), tc.data_ptr(),
                                             to.data_ptr())
        assert t["split"] in (2048, 4096, 6144, 8192, 10240, 12288, 14336, 16384, 32768)
        assert t["cell_factor"] in (0.5, 1.0, 2.0) and t["best_ms"] > 0
        got, st = clipper.clip_pairwise(base, ovs)
        assert (st == 0).all()
        assert all(rings_equal(a, b) for a, b in zip(got, ref))
    finally:
        clipper.set_pairwise_split(8192)
        clipper.set_pairwise_cell_factor(1.0)


def test_pairwise_special_overlays(clipper):
    base = gen.jagged_star(3_000, 3300, R=1000.0)
    b0 = base[0]
    ovs = []
    # a square across the boundary near vertex 0, and the same square sharing
    # base vertex 0's x value (leaves the rank shortcut)
    sq = np.array([[-30.0, -30.0], [30.0, -30.0], [30.0, 30.0], [-30.0, 30.0]])
    ovs.append(sq * [1.0, 0.9] + b0 + [0.37, 0.11])
    shared = sq + b0 + [0.0, 0.5]
    shared[0, 0] = b0[0]
    ovs.append(shared)
    # an axis-aligned rectangle (vertical edges)
    ovs.append(np.array([[0.0, 0.0], [200.0, 0.0], [200.0, 120.0], [0.0, 120.0]]) + b0 * 0.5)
    # far outside, deep inside, and an overlay containing the whole base
    ovs.append(gen.star(40, 1, centre=(5000.0, 5000.0), R=10.0))
    ovs.append(gen.star(400, 2, centre=(1.0, 2.0), R=20.0))
    ovs.append(gen.star(64, 3, centre=(0.5, -0.25), R=4000.0))
    # larger than the base, crossing it
    ovs.append(gen.star(4_000, 4, centre=(300.0, -200.0), R=900.0))
    # too short
    ovs.append(np.array([[0.0, 0.0], [1.0, 1.0]]))
    # triangles straddling many base edges
    for k in range(8):
        v = base[(k * 373) % len(base)]
        ovs.append(np.array([[v[0] - 40, v[1] - 35], [v[0] + 45, v[1] - 20], [v[0], v[1] + 50]]))
    _check(clipper, base, ovs)
    assert clipper.pairwise_info()["fallback_pairs"] >= 2


def test_pairwise_small_base_and_repeat(clipper):
    base = gen.star(12, 77, R=1.0)
    ovs = [gen.star(int(n), 100 + n, centre=(0.1 * n % 1 - 0.5, 0.05 * n % 1 - 0.5), R=0.6)
           for n in range(3, 40)]
    a = _check(clipper, base, ovs)
    b, _ = clipper.clip_pairwise(base, ovs)
    assert all(rings_equal(x, y) for x, y in zip(a, b))
    got, st = clipper.clip_pairwise(base, [])
    assert got == [] and len(st) == 0


def test_pairwise_area_and_gradient(clipper):
    """Areas against the FP64 shoelace of the oracle's rings, gradients against
    the host FP64 gradient of the same rings (base gradient summed over the
    overlays), 1e-12 relative; a fallback pair (shared x value) included."""
    torch = pytest.importorskip("torch")
    import area_grad as AG
    import sbclip
    base, ovs = gen.one_to_many(n_base=1_500, n_overlays=40, seed=3500, hi=300,
                                near_boundary=0.7)
    sq = np.array([[-30.0, -30.0], [30.0, -30.0], [30.0, 30.0], [-30.0, 30.0]]) + base[5]
    sq[1, 0] += 0.37
    sq[0, 0] = base[5, 0]  # shares an x value with the base: the pair pipeline clips it
    ovs.append(sq)
    cxy, coff = sbclip.pack_polygons(ovs)
    dev = "cuda:0"
    tb = torch.from_numpy(np.ascontiguousarray(base)).to(dev)
    tc = torch.from_numpy(cxy).to(dev)
    to = torch.from_numpy(coff).to(dev)
    n = len(ovs)
    area = torch.zeros(n, dtype=torch.float64, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    args = (tb.data_ptr(), len(base), n, tc.data_ptr(), to.data_ptr())
    clipper.pairwise_area_device(*args, area.data_ptr(), st.data_ptr())
    assert (st == 0).all()
    assert clipper.pairwise_info()["fallback_pairs"] >= 1
    w = torch.linspace(0.5, 2.0, n, dtype=torch.float64, device=dev)
    gb = torch.zeros_like(tb)
    gc = torch.zeros_like(tc)
    clipper.pairwise_area_backward_device(*args, w.data_ptr(), gb.data_ptr(), gc.data_ptr())
    a = area.cpu().numpy()
    gb, gc = gb.cpu().numpy(), gc.cpu().numpy()
    wb = np.zeros_like(base)
    for i, c in enumerate(ovs):
        want, hb, hc = AG.area_gradient(base, c)
        assert abs(a[i] - want) <= 1e-12 * max(1.0, abs(want)), i
        wb += w[i].item() * hb
        scale = max(np.abs(hc).max(), 1e-300) * w[i].item()
        assert np.abs(gc[coff[i]:coff[i + 1]] - w[i].item() * hc).max() <= 1e-11 * scale, i
    assert np.abs(gb - wb).max() <= 1e-11 * max(np.abs(wb).max(), 1e-300)


def test_pairwise_touching_overlays(clipper):
    """Overlays that touch the base exactly (vertices on its edges, an edge lying
    along one of its edges, bounces from either side) without sharing an x value
    with it, so they stay on the batched path: their labels take the rare
    branches (chains of overlapping edges, bouncing vertices, split pairs).
    Results and statuses must equal sbc_clip_pair's."""
    import sbclip
    base = np.array([[0.0, -8.0], [6.0, -6.0], [8.0, 0.0], [6.0, 6.0], [0.0, 8.0],
                     [-6.0, 6.0], [-8.0, 0.0], [-6.0, -6.0]])
    # edge (0,-8)-(6,-6): y = -8 + x/3; edge (6,-6)-(8,0): y = -6 + 3 (x - 6)
    on1 = lambda x: [x, -8.0 + x / 3.0]
    on2 = lambda x: [x, -6.0 + 3.0 * (x - 6.0)]
    ovs = [
        np.array([[2.0, -9.0], on1(3.0), [4.0, -9.5]]),             # bounce from outside
        np.array([[2.0, -5.0], [4.0, -5.5], on1(3.0)]),             # bounce from inside
        np.array([on1(1.5), on1(4.5), [4.5, -4.0], [1.5, -5.0]]),   # edge along the base's, inside
        np.array([on1(1.5), on1(4.5), [4.5, -9.0], [1.5, -9.5]]),   # the same, outside
        np.array([on1(1.5), on1(4.5), [4.5, -4.0], [2.5, -9.5]]),   # shared edge, then across
        np.array([on1(3.0), [7.5, -7.5], on2(7.0)]),                # a corner outside the base
        np.array([on1(3.0), on2(7.0), [4.5, -3.0]]),                # a corner cut inside
        np.array([on1(1.5), on1(3.0), [2.25, -10.0]]),              # two vertices on one edge
        np.array([[-1.0, -9.0], on1(3.0), [5.0, -9.0], [5.0, -4.0], [-1.0, -4.0]]),
    ]
    ovs += [o + [0.0, 0.0] for o in ovs[:4]]  # repeats in one call
    got, st = clipper.clip_pairwise(base, ovs)
    assert len(got) == len(ovs)
    for i, c in enumerate(ovs):
        try:
            want = clipper.clip_pair(base, c)
        except sbclip.SbcError as e:
            assert st[i] == e.code, (i, st[i], e.code)
            continue
        assert st[i] == 0, (i, st[i])
        assert rings_equal(got[i], want), i
    assert clipper.pairwise_info()["fallback_pairs"] < len(ovs)
