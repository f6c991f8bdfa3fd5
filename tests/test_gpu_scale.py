"""GPU parity of the batched paths at the sizes of their benchmark workloads,
and finite-difference checks of every gradient path.

* One base against many overlays: the whole 200,000-vertex base x 10,000
  overlays job (the bench's one_to_many_200k_10000 inputs) through
  sbc_clip_pairwise; rings bit for bit against the oracle on 120 overlays
  spread over the size range and against sbc_clip_pair on 1,000 seeded
  overlays; areas (1e-12) and gradients (1e-11, the pairwise backward adds
  with atomics) against the host FP64 gradient of the oracle's rings.
* Uneven many-pair batch: the 16 pairs of 200,000 vertices of the
  uneven_pairs_1m workload (same seeds) inside a batch of small uneven
  pairs; rings against the oracle, areas and gradients against the host FP64
  gradient of the oracle's rings.
* Finite differences, h = 1e-7 (scaled by the polygons' size where they are
  not unit-sized), central: 50 small pairs of 4-64 vertices (every
  coordinate), 2 pairs above the per-thread limit (the large-pair provenance
  path; sampled coordinates) and 5 overlays of the pairwise gradient (every
  overlay coordinate and sampled base coordinates).  The areas of the
  perturbed inputs are the exact shoelace sums of the GPU's output rings
  (area_grad.exact_shoelace), so the differences carry no FP64 summation
  noise; the step is the exact difference of the perturbed coordinates.
  Bar: max |analytic - FD| <= 1e-8 x max |analytic|.
* The pairwise engine's big-pair path with several worker threads against
  the oracle directly.
* The large jagged generator at R = 1 (where the reference's absolute
  EPSILON makes its trace undefined) at 50,000 vertices: the library returns
  SBC_EUNDEF, as the oracle does, in bounded time and memory.
"""
from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import area_grad as AG
import oracle_py as O
import sbclip_gen as gen
from conftest import rings_equal

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

FD_TOL = 1e-8


@pytest.fixture(scope="module")
def cl():
    import sbclip
    c = sbclip.Clipper(0)
    yield c
    c.close()


def _spread(sizes, n):
    """n indices whose sizes are evenly spaced ranks of the size order."""
    order = np.argsort(np.asarray(sizes), kind="stable")
    ranks = np.unique(np.linspace(0, len(order) - 1, n).round().astype(np.int64))
    return [int(order[r]) for r in ranks]


def _oracle_runs(pairs):
    """For every (base, overlay): (status, rings, area, grad_b, grad_c) of the
    oracle, on all host threads."""
    def one(p):
        b, c = p
        try:
            ov = O.clip(b, [c])["overlays"][0]
        except O.OracleError as e:
            return e.status, [], 0.0, None, None
        rings = O.rings_of(ov)
        a, gb, gc = AG.gradient_of_rings(b, c, rings, ov["uniq_b"], ov["uniq_c"], ov["uniq_t"],
                                         ov["isect_xy"])
        return 0, rings, a, gb, gc

    O.lib()
    with ThreadPoolExecutor() as ex:
        return list(ex.map(one, pairs))


def _device(torch, a, dtype=None):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to("cuda:0")


def test_one_to_many_200k_10000_matches_oracle(cl):
    torch = pytest.importorskip("torch")
    import sbclip
    base, ovs = gen.one_to_many()
    got, st = cl.clip_pairwise(base, ovs)
    info = cl.pairwise_info()
    assert (st == 0).all(), np.flatnonzero(st)[:8]
    assert info["unique"] > 100_000, info
    sample = _spread([len(o) for o in ovs], 120)
    runs = _oracle_runs([(base, ovs[i]) for i in sample])
    for i, (s, rings, *_rest) in zip(sample, runs):
        assert s == 0, (i, s)
        assert rings_equal(got[i], rings), i
    pick = np.random.default_rng(7).choice(len(ovs), 1000, replace=False)
    bad = [int(i) for i in pick if not rings_equal(got[i], cl.clip_pair(base, ovs[i]))]
    assert not bad, bad[:8]
    # areas of every overlay; gradients with the area weights of 40 sampled
    # overlays (the base gradient is summed over them, the others get none)
    cxy, coff = sbclip.pack_polygons(ovs)
    tb, tc, to = _device(torch, base), _device(torch, cxy), _device(torch, coff)
    n = len(ovs)
    area = torch.zeros(n, dtype=torch.float64, device="cuda:0")
    ast = torch.zeros(n, dtype=torch.int32, device="cuda:0")
    args = (tb.data_ptr(), len(base), n, tc.data_ptr(), to.data_ptr())
    cl.pairwise_area_device(*args, area.data_ptr(), ast.data_ptr())
    assert (ast == 0).all()
    a = area.cpu().numpy()
    for i, (_s, _r, want, _gb, _gc) in zip(sample, runs):
        assert abs(a[i] - want) <= 1e-12 * max(1.0, abs(want)), i
    wsel = sample[::3]
    w = np.zeros(n)
    w[wsel] = np.linspace(0.5, 2.0, len(wsel))
    tw = _device(torch, w)
    gb = torch.zeros_like(tb)
    gc = torch.zeros_like(tc)
    cl.pairwise_area_backward_device(*args, tw.data_ptr(), gb.data_ptr(), gc.data_ptr())
    gb, gc = gb.cpu().numpy(), gc.cpu().numpy()
    by_i = dict(zip(sample, runs))
    wb = np.zeros_like(base)
    for i in wsel:
        _s, _r, _a, hb, hc = by_i[i]
        wb += w[i] * hb
        scale = max(np.abs(hc).max(), 1e-300) * w[i]
        assert np.abs(gc[coff[i]:coff[i + 1]] - w[i] * hc).max() <= 1e-11 * scale, i
    assert np.abs(gb - wb).max() <= 1e-11 * max(np.abs(wb).max(), 1e-300)
    others = np.ones(n, bool)
    others[wsel] = False
    rows = np.repeat(others, np.diff(coff))
    assert not gc[rows].any()


def test_uneven_batch_large_pairs_match_oracle(cl):
    """The uneven_pairs_1m workload's 16 pairs of 200,000 vertices (same
    seeds), inside a batch of 4,000 uneven small pairs: through the large-pair
    path with the chunked arenas of the small ones."""
    bxy, boff, cxy, coff = gen.uneven_pairs(n_pairs=4_000, n_large=16)
    n = len(boff) - 1
    bases = [bxy[boff[p]:boff[p + 1]] for p in range(n)]
    ovs = [cxy[coff[p]:coff[p + 1]] for p in range(n)]
    large = [p for p in range(n) if len(bases[p]) == 200_000]
    assert len(large) == 16
    rings, st = cl.clip_batch(bases, ovs)
    assert cl.batch_info()["large_pairs"] == 16
    small = [int(p) for p in np.random.default_rng(11).choice(
        [p for p in range(n) if p not in large], 300, replace=False)]
    check = large + small
    runs = _oracle_runs([(bases[p], ovs[p]) for p in check])
    for p, (s, want, *_rest) in zip(check, runs):
        assert st[p] == s, (p, st[p], s)
        assert rings_equal(rings[p], want), p
    area, ast = cl.area_forward(bases, ovs)
    assert np.array_equal(ast, st)
    ga = np.random.default_rng(12).uniform(0.5, 2.0, n)
    gb, gc = cl.area_backward(bases, ovs, ga)
    for p, (s, _w, want, hb, hc) in zip(check, runs):
        if s != 0:
            continue
        assert abs(area[p] - want) <= 1e-12 * max(1.0, abs(want)), p
        scale = max(np.abs(hb).max(), np.abs(hc).max(), 1e-300) * ga[p]
        tol = (1e-11 if p in large else 1e-12) * scale  # large pairs add with atomics
        assert np.abs(gb[p] - ga[p] * hb).max() <= tol, p
        assert np.abs(gc[p] - ga[p] * hc).max() <= tol, p


def _fd_batch(cl, pairs, coords, h):
    """Central differences of the exact shoelace area of the GPU's rings.
    coords: per pair, a list of (polygon 0/1, vertex, axis).  Returns per pair
    the FD values in coords order."""
    bases, ovs, meta = [], [], []
    for p, (b, c) in enumerate(pairs):
        for which, i, k in coords[p]:
            for s in (1.0, -1.0):
                q = (b if which == 0 else c).copy()
                q[i, k] = q[i, k] + s * h
                bases.append(q if which == 0 else b)
                ovs.append(q if which == 1 else c)
            step = (bases[-2] if which == 0 else ovs[-2])[i, k] - \
                   (bases[-1] if which == 0 else ovs[-1])[i, k]
            meta.append((p, step))
    rings, st = cl.clip_batch(bases, ovs)
    assert (st == 0).all()
    out = [[] for _ in pairs]
    for j, (p, step) in enumerate(meta):
        ap = AG.exact_shoelace(rings[2 * j])
        am = AG.exact_shoelace(rings[2 * j + 1])
        out[p].append((ap - am) / step)
    return out


def _analytic(gb, gc, coords):
    return np.array([(gb if w == 0 else gc)[i, k] for w, i, k in coords])


def test_fd_small_pairs_every_coordinate(cl):
    """50 pairs of the small-pair workload's generator (4-64 vertices), every
    coordinate of both polygons."""
    pairs = gen.small_pairs(50, seed=4800)
    coords = [[(w, i, k) for w, P in ((0, b), (1, c)) for i in range(len(P)) for k in range(2)]
              for b, c in pairs]
    gb, gc = cl.area_backward([b for b, _ in pairs], [c for _, c in pairs], np.ones(len(pairs)))
    fd = _fd_batch(cl, pairs, coords, 1e-7)
    worst = 0.0
    for p in range(len(pairs)):
        an = _analytic(gb[p], gc[p], coords[p])
        if not np.abs(an).max() > 0:
            assert np.abs(fd[p]).max() == 0.0
            continue
        err = np.abs(an - fd[p]).max() / np.abs(an).max()
        worst = max(worst, err)
    assert worst <= FD_TOL, worst


def _sample_coords(rng, gb, gc, n):
    """n coordinates per polygon: half among vertices with a non-zero
    gradient (vertices that shape the result), half anywhere."""
    out = []
    for w, g in ((0, gb), (1, gc)):
        live = np.flatnonzero(np.abs(g).max(axis=1) > 0)
        pick = list(rng.choice(live, min(n // 2, len(live)), replace=False)) if len(live) else []
        pick += list(rng.choice(len(g), n - len(pick), replace=False))
        out += [(w, int(i), int(rng.integers(0, 2))) for i in pick]
    return out


def test_fd_large_pairs_provenance_path(cl):
    """Two pairs above the per-thread vertex limit: the pair pipeline clips
    them and the backward pass finds each ring vertex's provenance."""
    import sbclip
    big = sbclip.BATCH_MAX_VERTICES + 904
    pairs = [(gen.star(big, 4900), gen.star(big - 400, 4901, centre=(0.2, -0.1))),
             (gen.jagged_star(big + 100, 4902), gen.star(600, 4903, centre=(0.3, 0.25), R=0.5))]
    gb, gc = cl.area_backward([b for b, _ in pairs], [c for _, c in pairs], np.ones(2))
    assert cl.batch_info()["large_pairs"] == 2
    rng = np.random.default_rng(4904)
    coords = [_sample_coords(rng, gb[p], gc[p], 24) for p in range(2)]
    fd = _fd_batch(cl, pairs, coords, 1e-7)
    for p in range(2):
        an = _analytic(gb[p], gc[p], coords[p])
        assert np.abs(an).max() > 0
        assert np.abs(an - fd[p]).max() <= FD_TOL * np.abs(an).max(), p


def test_fd_pairwise_overlays_and_base(cl):
    """The pairwise gradient of 5 overlays crossing a 3,000-vertex jagged base
    (unit size): every overlay coordinate, and 24 sampled base coordinates
    against the summed areas of all 5."""
    torch = pytest.importorskip("torch")
    import sbclip
    h = 1e-7
    base = gen.jagged_star(3_000, 5100)
    rng = np.random.default_rng(5101)
    ovs = [gen.star(int(rng.integers(40, 121)), 5110 + j,
                    centre=tuple(base[int(rng.integers(0, len(base)))]),
                    R=float(rng.uniform(0.2, 0.4))) for j in range(5)]
    cxy, coff = sbclip.pack_polygons(ovs)
    tb, tc, to = _device(torch, base), _device(torch, cxy), _device(torch, coff)
    n = len(ovs)
    args = (tb.data_ptr(), len(base), n, tc.data_ptr(), to.data_ptr())
    area = torch.zeros(n, dtype=torch.float64, device="cuda:0")
    ast = torch.zeros(n, dtype=torch.int32, device="cuda:0")
    cl.pairwise_area_device(*args, area.data_ptr(), ast.data_ptr())
    assert (ast == 0).all() and (area.cpu().numpy() > 0).all()
    ones = torch.ones(n, dtype=torch.float64, device="cuda:0")
    gb = torch.zeros_like(tb)
    gc = torch.zeros_like(tc)
    cl.pairwise_area_backward_device(*args, ones.data_ptr(), gb.data_ptr(), gc.data_ptr())
    gb, gc = gb.cpu().numpy(), gc.cpu().numpy()
    # every overlay coordinate: the perturbed overlays of one call
    pert, meta = [], []
    for j, c in enumerate(ovs):
        for i in range(len(c)):
            for k in range(2):
                qp, qm = c.copy(), c.copy()
                qp[i, k] += h
                qm[i, k] -= h
                pert += [qp, qm]
                meta.append((j, i, k, qp[i, k] - qm[i, k]))
    rings, st = cl.clip_pairwise(base, pert)
    assert (st == 0).all()
    for j in range(n):
        an, fd = [], []
        for t, (jj, i, k, step) in enumerate(meta):
            if jj != j:
                continue
            an.append(gc[coff[j] + i, k])
            fd.append((AG.exact_shoelace(rings[2 * t]) - AG.exact_shoelace(rings[2 * t + 1])) / step)
        an, fd = np.array(an), np.array(fd)
        assert np.abs(an - fd).max() <= FD_TOL * np.abs(an).max(), j
    # sampled base coordinates: the summed areas of all overlays
    live = np.flatnonzero(np.abs(gb).max(axis=1) > 0)
    picks = list(rng.choice(live, min(16, len(live)), replace=False))
    picks += list(rng.choice(len(base), 8, replace=False))
    an, fd = [], []
    for i in picks:
        k = int(rng.integers(0, 2))
        bp, bm = base.copy(), base.copy()
        bp[i, k] += h
        bm[i, k] -= h
        rp, sp = cl.clip_pairwise(bp, ovs)
        rm, sm = cl.clip_pairwise(bm, ovs)
        assert (sp == 0).all() and (sm == 0).all()
        ap = sum(AG.exact_shoelace(r) for r in rp)
        am = sum(AG.exact_shoelace(r) for r in rm)
        an.append(gb[i, k])
        fd.append((ap - am) / (bp[i, k] - bm[i, k]))
    an, fd = np.array(an), np.array(fd)
    assert np.abs(an).max() > 0
    assert np.abs(an - fd).max() <= FD_TOL * np.abs(an).max()


def test_pairwise_big_pairs_on_several_workers_match_oracle(cl):
    """A split of 64 records sends most overlays to the data-parallel rows,
    shared by the big-pair worker threads; every overlay's rings against the
    oracle directly."""
    base, ovs = gen.one_to_many(n_base=20_000, n_overlays=48, seed=3700, hi=2000,
                                near_boundary=0.8)
    workers = cl.pairwise_workers()
    try:
        cl.set_pairwise_split(64)
        got, st = cl.clip_pairwise(base, ovs)
        info = cl.pairwise_info()
        cl.set_pairwise_workers(3)
        got3, st3 = cl.clip_pairwise(base, ovs)
    finally:
        cl.set_pairwise_split(8192)
        cl.set_pairwise_workers(workers)
    assert info["big_pairs"] >= 16, info
    runs = _oracle_runs([(base, c) for c in ovs])
    for i, (s, want, *_rest) in enumerate(runs):
        assert st[i] == s and st3[i] == s, (i, st[i], st3[i], s)
        assert rings_equal(got[i], want) and rings_equal(got3[i], want), i


def test_jagged_pair_at_unit_radius_fails_cleanly():
    """At R = 1 the jagged generator's tangential edges give cross products
    below the reference's absolute EPSILON (1e-9), collinear chains follow
    and the reference's result is undefined (its trace grows without bound).
    At 50,000 vertices the oracle returns its 'undefined' status; the library
    must return SBC_EUNDEF too, in bounded time and device memory, and the
    context must stay usable."""
    torch = pytest.importorskip("torch")
    import sbclip
    b, c = gen.pair_large(50_000, R=1.0)
    with pytest.raises(O.OracleError) as oe:
        O.clip(b, [c])
    assert oe.value.status == 2
    clipper = sbclip.Clipper(0)
    try:
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        t0 = time.time()
        with pytest.raises(sbclip.SbcError) as e:
            clipper.clip_pair(b, c)
        elapsed = time.time() - t0
        used = free0 - torch.cuda.mem_get_info(0)[0]
        assert e.value.code == 2, str(e.value)
        assert elapsed < 60.0, elapsed
        assert used < (4 << 30), used
        # the context stays usable
        b2, c2 = gen.pair_large(50_000)
        assert rings_equal(clipper.clip_pair(b2, c2), O.rings_of(O.clip(b2, [c2])["overlays"][0]))
    finally:
        clipper.close()
