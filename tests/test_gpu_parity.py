"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's golden outputs.  Integer and index results are compared for
equality and FP64 results bit for bit (no tolerance: the reference's output
rings must be reproduced exactly)."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_py as O
import sbclip_gen as gen
from conftest import KAT_PAIRS, digest, ring_digest, rings_equal

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_classifier_known_answers(clipper):
    pairs = np.array([[*p1, *p2, *q1, *q2] for p1, p2, q1, q2, _ in KAT_PAIRS], float)
    t, a, b, ai, bi = clipper.classify(pairs)
    assert list(t) == [w for *_, w in KAT_PAIRS]


def test_classifier_matches_oracle_random(clipper):
    rng = np.random.default_rng(5)
    n = 20000
    pairs = rng.uniform(-1, 1, (n, 8))
    # make a share of the pairs touch or overlap (degenerate types)
    pairs[: n // 4, 4:6] = pairs[: n // 4, 0:2]
    pairs[n // 4: n // 2, 6:8] = pairs[n // 4: n // 2, 0:2] * 2 - pairs[n // 4: n // 2, 2:4]
    t, a, b, _, _ = clipper.classify(pairs)
    for i in range(0, n, 7):
        ot, oa, ob = O.segment_intersection(pairs[i, 0:2], pairs[i, 2:4], pairs[i, 4:6], pairs[i, 6:8])
        assert t[i] == ot
        if ot:
            assert a[i] == oa and b[i] == ob


def test_small_cases_match_reference(clipper, small_cases):
    for case in small_cases:
        got = clipper.clip(case.base, case.overlays)
        for i in range(len(case.overlays)):
            assert rings_equal(got[i], case.rings[i]), case.kind


def test_small_cases_serial_back_end_matches(small_cases):
    import sbclip
    c = sbclip.Clipper(0, serial_backend=True)
    try:
        for case in small_cases:
            got = c.clip(case.base, case.overlays)
            for i in range(len(case.overlays)):
                assert rings_equal(got[i], case.rings[i]), case.kind
    finally:
        c.close()


def test_small_cases_tree_stages_match_oracle(clipper, small_cases):
    """Rows A4-A7 (elementary points, end lists, cover lists) on every small
    case, degenerate grids and vertical edges included."""
    for case in small_cases:
        clipper.clip(case.base, case.overlays)
        _check_tree(clipper, O.clip(case.base, case.overlays))


def test_unique_pairs_match_reference(clipper, small_cases):
    for case in small_cases:
        if len(case.overlays) != 1:
            continue
        clipper.clip(case.base, case.overlays)
        ub, uc, ut = case.uniq[0]
        assert np.array_equal(clipper.debug_array("uniq_b"), ub)
        assert np.array_equal(clipper.debug_array("uniq_c"), uc)
        assert np.array_equal(clipper.debug_array("uniq_t"), ut)


def _cover_pairs(lr, L):
    """(node, edge) pairs of every edge's canonical decomposition of its leaf
    range [l, r1): the nodes the reference's insertEdgeParallel
    (p_seg_tree/oacc_segment_tree.cpp:2496-2564) puts the edge in."""
    e = np.arange(len(lr), dtype=np.int64)
    x = lr[:, 0].astype(np.int64) + L
    y = lr[:, 1].astype(np.int64) + L
    nodes, edges = [], []
    while True:
        live = x < y
        if not live.any():
            break
        a = live & (x & 1 == 1)
        nodes.append(x[a]); edges.append(e[a])
        x = np.where(a, x + 1, x)
        b = live & (y & 1 == 1)
        y = np.where(b, y - 1, y)
        nodes.append(y[b]); edges.append(e[b])
        x >>= 1
        y >>= 1
    nodes = np.concatenate(nodes) if nodes else np.zeros(0, np.int64)
    edges = np.concatenate(edges) if edges else np.zeros(0, np.int64)
    o = np.lexsort((edges, nodes))
    return nodes[o], edges[o]


def _check_tree(clipper, ora):
    """Rows A4-A7 directly: the elementary points bit for bit, every leaf's
    end list and every node's cover list entry for entry, and the counts."""
    st, t, s = clipper.stats(), ora["tree"], ora["stats"]
    assert st["elementary_points"] == s["elem_count"]
    assert st["tree_size"] == s["tree_size"]
    assert st["cover_entries"] == s["cover_total"]
    assert st["leaf_end_entries"] == s["leaf_end_total"]
    ea = clipper.debug_array("elementary")
    assert np.array_equal(ea.view(np.int64), t["ea"].view(np.int64))
    L = s["tree_size"] // 2
    aft = clipper.debug_array("leaf_after").astype(np.int64)
    bef = clipper.debug_array("leaf_before").astype(np.int64)
    E = len(aft)
    assert E == s["edges"] == len(bef)
    # A6: leaf q lists, in edge order, each edge's end entry, then its start entry
    e = np.arange(E, dtype=np.int64)
    leaf = np.concatenate([aft, bef])
    ent = np.concatenate([e, e])
    kind = np.concatenate([np.zeros(E, np.int64), np.ones(E, np.int64)])
    ok = leaf >= 0
    leaf, ent, kind = leaf[ok] - L, ent[ok], kind[ok]
    o = np.lexsort((kind, ent, leaf))
    assert np.array_equal(ent[o], t["leaf_edge"])
    assert np.array_equal(np.searchsorted(leaf[o], np.arange(L + 1)), t["leaf_off"])
    # A7: node v's cover list, ascending edge index
    lr = clipper.debug_array("leaf_range").reshape(-1, 2)
    nodes, edges = _cover_pairs(lr, L)
    assert np.array_equal(edges, t["cov_edge"])
    assert np.array_equal(np.searchsorted(nodes, np.arange(2 * L + 1)), t["cov_off"])


def _compare_all(clipper, b, c, entry=None):
    rings = clipper.clip(b, [c])[0]
    run = O.clip(b, [c])
    ora = run["overlays"][0]
    _check_tree(clipper, run)
    assert clipper.stats()["raw_hits"] == len(ora["raw_b"])
    for name in ("uniq_b", "uniq_c", "uniq_t", "isect_ab", "isect_ac", "isect_xy",
                 "merged_bxy", "merged_cxy", "merged_balpha", "merged_calpha",
                 "merged_bnb", "merged_cnb", "label_b", "label_c"):
        g = clipper.debug_array(name)
        assert np.array_equal(g, ora[name].astype(g.dtype)), name
    assert rings_equal(rings, O.rings_of(ora))
    if entry is not None and digest(b, c) == entry["input_sha256"]:
        assert len(rings) == entry["rings"]
        assert ring_digest(rings) == entry["rings_sha256"]
    return rings


def test_pair_10k_8k_all_stages(clipper, digests):
    b, c = gen.pair_small()
    _compare_all(clipper, b, c, digests["pair_10k_8k"])
    st = clipper.stats()
    assert st["unique"] == digests["pair_10k_8k"]["unique"]
    assert st["serial_backend"] == 0


@pytest.mark.slow
def test_pair_1m_1m_all_stages(clipper, digests):
    b, c = gen.pair_large()
    _compare_all(clipper, b, c, digests["pair_1m_1m"])
    assert clipper.stats()["serial_backend"] == 0


def test_swapped_roles_and_jagged_mid_size(clipper):
    b, c = gen.pair_large(n=50_000)
    _compare_all(clipper, b, c)
    _compare_all(clipper, c, b)


def test_cli_text_matches_reference(tmp_path, digests):
    b, c = gen.pair_small()
    gen.write_poly(tmp_path / "b.txt", b)
    gen.write_poly(tmp_path / "c.txt", c)
    (tmp_path / "work").mkdir()
    (tmp_path / "results").mkdir()
    exe = ROOT / "segment-tree-based-clipping_gb300" / "_build" / "seg"
    p = subprocess.run([str(exe), str(tmp_path / "b.txt"), str(tmp_path / "c.txt")],
                       cwd=tmp_path / "work", capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    text = (tmp_path / "results" / "Fig-def-R1.txt").read_text()
    import hashlib
    assert hashlib.sha256(text.encode()).hexdigest() == digests["pair_10k_8k"]["text6_sha256"]


def test_errors_are_status_codes(clipper):
    import sbclip
    with pytest.raises(sbclip.SbcError) as e:
        clipper.clip(np.array([[0, 0], [1, 0]], float), [gen.star(5, 1)])
    assert e.value.code == 1
    bad = gen.star(10, 1)
    bad[3, 0] = np.nan
    with pytest.raises(sbclip.SbcError) as e:
        clipper.clip(bad, [gen.star(5, 2)])
    assert e.value.code == 1
    # the context stays usable after an error
    b, c = gen.star(40, 3), gen.star(30, 4, centre=(0.2, 0.1))
    assert rings_equal(clipper.clip(b, [c])[0], O.rings_of(O.clip(b, [c])["overlays"][0]))


def test_repeat_calls_are_identical(clipper):
    b, c = gen.pair_small()
    r1 = clipper.clip(b, [c])[0]
    r2 = clipper.clip(b, [c])[0]
    assert rings_equal(r1, r2)


def test_kernels_were_launched(clipper):
    import sbclip
    before = sbclip.kernel_launches()
    clipper.clip(gen.star(100, 1), [gen.star(80, 2, centre=(0.1, 0.1))])
    assert sbclip.kernel_launches() > before + 20


def _same_tree_arrays(a_clip, b_clip, tag):
    for name in ("elementary", "leaf_after", "leaf_before", "leaf_range"):
        a, w = a_clip.debug_array(name), b_clip.debug_array(name)
        assert np.array_equal(a.view(np.int64) if a.dtype == np.float64 else a,
                              w.view(np.int64) if w.dtype == np.float64 else w), (tag, name)


def test_vertex_sort_and_endpoint_sort_agree(clipper, small_cases):
    """The elementary intervals come from a sort of the E vertex keys,
    expanded to the 2E endpoints; inputs with a shared x value fall back to
    sorting the endpoints themselves.  The vertex sort runs on 32-bit keys
    with equal-key runs fixed up (stat 2), or on the 64-bit keys (stat 1, the
    wide_vertex_sort hook).  Every route gives the same tree arrays and
    rings."""
    import sbclip
    ref = sbclip.Clipper(0, endpoint_sort=True)
    wide = sbclip.Clipper(0, wide_vertex_sort=True)
    try:
        kinds = set()
        cases = [(c.kind, c.base, c.overlays) for c in small_cases]
        pb, pc = gen.pair_small()
        cases.append(("pair_10k_8k", pb, [pc]))
        for kind, b, ovs in cases:
            got = clipper.clip(b, ovs)
            vs = clipper.stats()["vertex_sort"]
            kinds.add(vs)
            want = ref.clip(b, ovs)
            assert ref.stats()["vertex_sort"] == 0
            _same_tree_arrays(clipper, ref, kind)
            got_w = wide.clip(b, ovs)
            assert wide.stats()["vertex_sort"] in (0, 1) and (vs == 0) == (
                wide.stats()["vertex_sort"] == 0), kind
            _same_tree_arrays(wide, ref, kind)
            for x, y, z in zip(got, want, got_w):
                assert rings_equal(x, y) and rings_equal(z, y), kind
        assert kinds == {0, 2}  # both routes ran
    finally:
        ref.close()
        wide.close()


def _near_vertical_chain(n: int):
    """A simple polygon whose right side is a chain of n vertices going up
    with x = 1 - i * 2^-50: distinct x values far closer together than the
    x range / 2^32, and falling with the vertex index, so one 32-bit key run
    holds them in reverse order."""
    d = 2.0 ** -50
    chain = [(1.0 - i * d, -0.9 + 1.8 * i / (n - 1)) for i in range(n)]
    pts = [(-1.0, -1.0), (0.97, -1.03)] + chain + [(0.96, 1.04), (-1.02, 0.99)]
    return np.array(pts, dtype=np.float64)


@pytest.mark.parametrize("n,stat", [(6, 2), (32, 2), (48, 1)])
def test_vertex_key_runs_are_fixed_up(clipper, n, stat):
    """Equal 32-bit vertex keys: runs of up to 32 vertices are put in full-key
    order in place (stat 2); a longer run sends the stage back to the 64-bit
    vertex sort (stat 1).  Every stage and the rings equal the oracle's and
    the endpoint sort's."""
    import sbclip
    b = _near_vertical_chain(n)
    c = gen.star(64, 71, centre=(0.95, 0.0), R=0.3)
    _compare_all(clipper, b, c)
    assert clipper.stats()["vertex_sort"] == stat
    ref = sbclip.Clipper(0, endpoint_sort=True)
    try:
        ref.clip(b, [c])
        _same_tree_arrays(clipper, ref, n)
    finally:
        ref.close()


def test_common_mbr_filter_keeps_every_candidate(clipper):
    """A small overlay against a large base: most base edges miss the common
    MBR of the two polygons and are left out of the candidate search; every
    stage and the rings still equal the oracle's (also with several overlays,
    and with an overlay whose box misses the base's entirely)."""
    b = gen.star(20_000, 61)
    c = gen.star(300, 62, centre=(0.55, 0.05), R=0.12)
    _compare_all(clipper, b, c)
    st = clipper.stats()
    assert st["outside_cmbr"] > 15_000, st
    far = gen.star(50, 63, centre=(5.0, 5.0), R=0.1)
    ovs = [c, gen.star(200, 64, centre=(-0.4, 0.3), R=0.2), far]
    got = clipper.clip(b, ovs)
    ora = O.clip(b, ovs)["overlays"]
    for i in range(len(ovs)):
        assert rings_equal(got[i], O.rings_of(ora[i])), i
    assert got[2] == []
