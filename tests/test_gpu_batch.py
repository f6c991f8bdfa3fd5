"""GPU checks of the batched entry points (sbc_clip_batch, sbc_area_forward,
sbc_area_backward and their device-array forms) through the C ABI.

Rings are compared bit for bit with the reference's golden rings and with
the oracle pair by pair; areas with the FP64 shoelace of the oracle's rings
to 1e-12 relative; gradients with the host FP64 gradient of the same rings
to 1e-12 relative and with central finite differences (h = 1e-7) of the GPU
area to 1e-8 relative."""
from __future__ import annotations

import numpy as np
import pytest

import area_grad as AG
import oracle_py as O
import sbclip_gen as gen
from conftest import load_small_cases, rings_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cl():
    import sbclip
    c = sbclip.Clipper(0)
    yield c
    c.close()


def test_batch_rings_match_golden_small_cases(cl):
    cases = [c for c in load_small_cases() if len(c.overlays) == 1]
    rings, st = cl.clip_batch([c.base for c in cases], [c.overlays[0] for c in cases])
    assert (st == 0).all()
    for case, got in zip(cases, rings):
        assert rings_equal(got, case.rings[0]), case.kind


def test_batch_small_pairs_match_oracle_and_pair_path(cl):
    pairs = gen.small_pairs(2000, seed=4000)
    rings, st = cl.clip_batch([b for b, _ in pairs], [c for _, c in pairs])
    assert (st == 0).all()
    for (b, c), got in zip(pairs, rings):
        want = O.rings_of(O.clip(b, [c])["overlays"][0])
        assert rings_equal(got, want)
    for (b, c), got in list(zip(pairs, rings))[:40]:
        assert rings_equal(got, cl.clip_pair(b, c))


def test_batch_area_matches_oracle_shoelace(cl):
    pairs = gen.small_pairs(500, seed=4100)
    area, st = cl.area_forward([b for b, _ in pairs], [c for _, c in pairs])
    assert (st == 0).all()
    for (b, c), a in zip(pairs, area):
        want = AG.area(b, c)
        assert abs(a - want) <= 1e-12 * max(1.0, abs(want))


def test_batch_gradient_matches_host_gradient(cl):
    pairs = gen.small_pairs(200, seed=4200)
    bases, ovs = [b for b, _ in pairs], [c for _, c in pairs]
    ga = np.random.default_rng(1).uniform(0.5, 2.0, len(pairs))
    gb, gc = cl.area_backward(bases, ovs, ga)
    for p, (b, c) in enumerate(pairs):
        _, hb, hc = AG.area_gradient(b, c)
        scale = max(np.abs(hb).max(), np.abs(hc).max(), 1e-300) * ga[p]
        assert np.abs(gb[p] - ga[p] * hb).max() <= 1e-12 * scale
        assert np.abs(gc[p] - ga[p] * hc).max() <= 1e-12 * scale


def test_batch_gradient_matches_finite_differences(cl):
    h = 1e-7
    for b, c in gen.small_pairs(3, seed=4300, lo=5, hi=20):
        gb, gc = cl.area_backward([b], [c], np.ones(1))
        # every +-h perturbation of every coordinate as one batch
        bases, ovs = [], []
        for which, P in ((0, b), (1, c)):
            for i in range(len(P)):
                for k in range(2):
                    for s in (1.0, -1.0):
                        q = P.copy()
                        q[i, k] += s * h
                        bases.append(q if which == 0 else b)
                        ovs.append(q if which == 1 else c)
        area, st = cl.area_forward(bases, ovs)
        assert (st == 0).all()
        fd = (area[0::2] - area[1::2]) / (2 * h)
        an = np.concatenate([gb[0].ravel(), gc[0].ravel()])
        a0, _ = cl.area_forward([b], [c])
        scale = max(np.abs(an).max(), abs(a0[0]))
        assert np.abs(an - fd).max() <= 1e-8 * scale


def test_batch_statuses_and_empty_batch(cl):
    import sbclip
    b, c = gen.star(20, 5), gen.star(10, 6, centre=(0.1, 0.1))
    tiny = np.array([[0.0, 0.0], [1.0, 0.0]])
    huge = gen.star(sbclip.BATCH_MAX_VERTICES + 1, 7)
    rings, st = cl.clip_batch([b, tiny, b, huge], [c, c, tiny, c])
    assert list(st) == [0, 1, 1, 0]
    assert rings[1] == [] and rings[2] == []
    assert rings_equal(rings[0], cl.clip_pair(b, c))
    assert rings_equal(rings[3], cl.clip_pair(huge, c))
    assert cl.batch_info()["large_pairs"] == 1
    area, st = cl.area_forward([], [])
    assert len(area) == 0


def _mixed(seed):
    """Small pairs with large ones (a polygon above the per-thread limit) mixed in."""
    import sbclip
    pairs = gen.small_pairs(300, seed=seed)
    big = sbclip.BATCH_MAX_VERTICES + 500
    pairs.insert(7, (gen.star(big, seed + 1), gen.star(300, seed + 2, centre=(0.2, -0.1))))
    pairs.insert(150, (gen.star(250, seed + 3), gen.star(big, seed + 4, centre=(-0.1, 0.15))))
    pairs.append((gen.star(big + 100, seed + 5), gen.star(big, seed + 6, centre=(0.3, 0.1))))
    return pairs


def test_batch_large_pairs_rings_areas_gradients(cl):
    pairs = _mixed(4500)
    bases, ovs = [b for b, _ in pairs], [c for _, c in pairs]
    rings, st = cl.clip_batch(bases, ovs)
    assert (st == 0).all()
    assert cl.batch_info()["large_pairs"] == 3
    for i in (7, 150, len(pairs) - 1, 0, 99):
        assert rings_equal(rings[i], cl.clip_pair(bases[i], ovs[i])), i
    area, st = cl.area_forward(bases, ovs)
    ga = np.random.default_rng(3).uniform(0.5, 2.0, len(pairs))
    gb, gc = cl.area_backward(bases, ovs, ga)
    for i in (7, 150, len(pairs) - 1):
        want = AG.area(bases[i], ovs[i])
        assert abs(area[i] - want) <= 1e-12 * max(1.0, abs(want)), i
        _, hb, hc = AG.area_gradient(bases[i], ovs[i])
        scale = max(np.abs(hb).max(), np.abs(hc).max(), 1e-300) * ga[i]
        assert np.abs(gb[i] - ga[i] * hb).max() <= 1e-12 * scale, i
        assert np.abs(gc[i] - ga[i] * hc).max() <= 1e-12 * scale, i


def test_batch_chunks_match_one_chunk(cl):
    """A tiny arena budget cuts the batch into many chunks; the backward pass
    then recomputes each chunk's forward.  Results equal the one-chunk run."""
    pairs = _mixed(4600)
    bases, ovs = [b for b, _ in pairs], [c for _, c in pairs]
    ga = np.random.default_rng(4).uniform(0.5, 2.0, len(pairs))
    r1, s1 = cl.clip_batch(bases, ovs)
    a1, _ = cl.area_forward(bases, ovs)
    gb1, gc1 = cl.area_backward(bases, ovs, ga)
    try:
        cl.set_batch_arena_budget(2 << 20)
        r2, s2 = cl.clip_batch(bases, ovs)
        assert cl.batch_info()["chunks"] > 5
        a2, _ = cl.area_forward(bases, ovs)
        gb2, gc2 = cl.area_backward(bases, ovs, ga)
    finally:
        cl.set_batch_arena_budget(0)
    assert np.array_equal(s1, s2) and np.array_equal(a1, a2)
    assert all(rings_equal(x, y) for x, y in zip(r1, r2))
    small = [i for i in range(len(pairs)) if i not in (7, 150, len(pairs) - 1)]
    for i in small:
        assert np.array_equal(gb1[i], gb2[i]) and np.array_equal(gc1[i], gc2[i]), i
    for i in (7, 150, len(pairs) - 1):
        assert np.allclose(gb1[i], gb2[i], rtol=1e-12, atol=1e-12 * np.abs(gb1[i]).max())


def test_batch_device_arrays_match_host_arrays(cl):
    torch = pytest.importorskip("torch")
    import sbclip
    pairs = gen.small_pairs(300, seed=4400)
    bases, ovs = [b for b, _ in pairs], [c for _, c in pairs]
    bxy, boff = sbclip.pack_polygons(bases)
    cxy, coff = sbclip.pack_polygons(ovs)
    dev = "cuda:0"
    t = {k: torch.from_numpy(v).to(dev) for k, v in
         (("bxy", bxy), ("boff", boff), ("cxy", cxy), ("coff", coff))}
    area = torch.zeros(len(pairs), dtype=torch.float64, device=dev)
    st = torch.zeros(len(pairs), dtype=torch.int32, device=dev)
    args = (len(pairs), t["bxy"].data_ptr(), t["boff"].data_ptr(), t["cxy"].data_ptr(),
            t["coff"].data_ptr())
    cl.area_forward_device(*args, area.data_ptr(), st.data_ptr())
    ga = torch.full((len(pairs),), 1.5, dtype=torch.float64, device=dev)
    gb = torch.zeros_like(t["bxy"])
    gc = torch.zeros_like(t["cxy"])
    cl.area_backward_device(*args, ga.data_ptr(), gb.data_ptr(), gc.data_ptr())
    h_area, h_st = cl.area_forward(bases, ovs)
    h_gb, h_gc = cl.area_backward(bases, ovs, np.full(len(pairs), 1.5))
    assert np.array_equal(area.cpu().numpy(), h_area)
    assert np.array_equal(st.cpu().numpy(), h_st)
    assert np.array_equal(gb.cpu().numpy(), np.concatenate(h_gb))
    assert np.array_equal(gc.cpu().numpy(), np.concatenate(h_gc))


def test_batch_area_graph_replays_forward_and_backward(cl):
    """One CUDA graph launch equals sbc_area_forward_device +
    sbc_area_backward_device, bit for bit, also after the coordinates change
    in place; a later batched call on the context makes the graph stale."""
    torch = pytest.importorskip("torch")
    import sbclip
    pairs = gen.small_pairs(500, seed=4700)
    bxy, boff = sbclip.pack_polygons([b for b, _ in pairs])
    cxy, coff = sbclip.pack_polygons([c for _, c in pairs])
    dev = "cuda:0"
    t = {k: torch.from_numpy(v).to(dev) for k, v in
         (("bxy", bxy), ("boff", boff), ("cxy", cxy), ("coff", coff))}
    n = len(pairs)
    args = (n, t["bxy"].data_ptr(), t["boff"].data_ptr(), t["cxy"].data_ptr(),
            t["coff"].data_ptr())
    ga = torch.linspace(0.5, 2.0, n, dtype=torch.float64, device=dev)
    out = {k: torch.zeros_like(t[s2]) for k, s2 in (("gb", "bxy"), ("gc", "cxy"))}
    area = torch.zeros(n, dtype=torch.float64, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    g = cl.area_graph(*args, ga.data_ptr(), out["gb"].data_ptr(), out["gc"].data_ptr(),
                      area.data_ptr(), st.data_ptr())
    ref = sbclip.Clipper(0)
    try:
        def reference():
            a = torch.zeros(n, dtype=torch.float64, device=dev)
            s_ = torch.zeros(n, dtype=torch.int32, device=dev)
            gb = torch.zeros_like(t["bxy"])
            gc = torch.zeros_like(t["cxy"])
            ref.area_forward_device(*args, a.data_ptr(), s_.data_ptr())
            ref.area_backward_device(*args, ga.data_ptr(), gb.data_ptr(), gc.data_ptr())
            return a, s_, gb, gc
        for _ in range(2):
            area.zero_()
            out["gb"].zero_()
            g.launch()
            torch.cuda.synchronize()
            a, s_, gb, gc = reference()
            assert torch.equal(area, a) and torch.equal(st, s_)
            assert torch.equal(out["gb"], gb) and torch.equal(out["gc"], gc)
            assert (s_ == 0).all()
        # new coordinates of the same polygons, in place: a uniform scaling
        # keeps every pair's combinatorics, so its hit room still fits
        t["bxy"].mul_(1.25)
        t["cxy"].mul_(1.25)
        g.launch()
        torch.cuda.synchronize()
        a, s_, gb, gc = reference()
        assert torch.equal(area, a) and torch.equal(out["gb"], gb) and torch.equal(out["gc"], gc)
        # a later batched call on the same context replaces the graph's buffers
        cl.area_forward([pairs[0][0]], [pairs[0][1]])
        with pytest.raises(sbclip.SbcError) as e:
            g.launch()
        assert e.value.code == 1
    finally:
        g.close()
        ref.close()


def test_batch_shape_and_autotune_do_not_change_results(cl):
    """Block sizes and the small/large split are tuning knobs: rings, areas and
    gradients are the same under any setting (a split of 40 sends the pairs
    with a polygon above 40 vertices through the single-pair pipeline), and
    the autotuner keeps a valid setting."""
    torch = pytest.importorskip("torch")
    import sbclip
    pairs = gen.small_pairs(400, seed=4900)
    bases, ovs = [b for b, _ in pairs], [c for _, c in pairs]
    ga = np.random.default_rng(5).uniform(0.5, 2.0, len(pairs))
    r0, s0 = cl.clip_batch(bases, ovs)
    a0, _ = cl.area_forward(bases, ovs)
    gb0, gc0 = cl.area_backward(bases, ovs, ga)
    default = cl.batch_shape()
    try:
        cl.set_batch_shape(front=32, cand=64, back=32, backward=64, split=40)
        r1, s1 = cl.clip_batch(bases, ovs)
        assert cl.batch_info()["large_pairs"] > 50
        a1, _ = cl.area_forward(bases, ovs)
        gb1, gc1 = cl.area_backward(bases, ovs, ga)
        assert np.array_equal(s0, s1)
        assert all(rings_equal(x, y) for x, y in zip(r0, r1))
        # the single-pair path sums areas in two stages and gradients with atomics
        assert np.all(np.abs(a0 - a1) <= 1e-12 * np.maximum(1.0, np.abs(a0)))
        for p in range(len(pairs)):
            sc = max(np.abs(gb0[p]).max(), np.abs(gc0[p]).max(), 1e-300)
            assert np.abs(gb0[p] - gb1[p]).max() <= 1e-11 * sc, p
            assert np.abs(gc0[p] - gc1[p]).max() <= 1e-11 * sc, p
        cl.set_batch_shape(**default)
        bxy, boff = sbclip.pack_polygons(bases)
        cxy, coff = sbclip.pack_polygons(ovs)
        t = {k: torch.from_numpy(v).to("cuda:0") for k, v in
             (("bxy", bxy), ("boff", boff), ("cxy", cxy), ("coff", coff))}
        tga = torch.from_numpy(ga).to("cuda:0")
        gb = torch.zeros_like(t["bxy"])
        gc = torch.zeros_like(t["cxy"])
        tuned = cl.autotune_batch_device(len(pairs), t["bxy"].data_ptr(), t["boff"].data_ptr(),
                                         t["cxy"].data_ptr(), t["coff"].data_ptr(),
                                         tga.data_ptr(), gb.data_ptr(), gc.data_ptr())
        assert tuned["best_ms"] > 0
        assert all(tuned[k] in (32, 64, 128) for k in ("front", "cand", "back", "backward"))
        assert tuned["split"] == sbclip.BATCH_MAX_VERTICES  # no pair above 64 vertices
        r2, s2 = cl.clip_batch(bases, ovs)
        a2, _ = cl.area_forward(bases, ovs)
        assert np.array_equal(s0, s2) and np.array_equal(a0, a2)
        assert all(rings_equal(x, y) for x, y in zip(r0, r2))
    finally:
        cl.set_batch_shape(**default)
