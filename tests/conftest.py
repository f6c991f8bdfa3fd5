"""Shared test configuration: import paths, the `gpu` marker, fixtures."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "segment-tree-based-clipping_gb300"
for p in (ROOT / "oracle", PKG, ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: runs longer than a few seconds")


class SmallCase:
    def __init__(self, kind, base, overlays, rings, uniq):
        self.kind, self.base, self.overlays, self.rings, self.uniq = kind, base, overlays, rings, uniq


def load_small_cases():
    z = np.load(GOLDEN / "golden_small.npz")
    cases = []
    ci = ri = ro = ui = 0
    for i, kind in enumerate(z["kind"]):
        b = z["b_xy"][z["b_off"][i]:z["b_off"][i + 1]]
        k = int(z["c_cnt"][i])
        ovs, rings, uniq = [], [], []
        for _ in range(k):
            ovs.append(z["c_xy"][z["c_off"][ci]:z["c_off"][ci + 1]])
            ci += 1
            nr = int(z["r_ring_cnt"][ri])
            ri += 1
            rr = []
            for _ in range(nr):
                rr.append(z["r_xy"][z["r_off"][ro]:z["r_off"][ro + 1]])
                ro += 1
            rings.append(rr)
            a, bnd = z["u_off"][ui], z["u_off"][ui + 1]
            uniq.append((z["u_b"][a:bnd], z["u_c"][a:bnd], z["u_t"][a:bnd]))
            ui += 1
        cases.append(SmallCase(str(kind), b, ovs, rings, uniq))
    return cases


@pytest.fixture(scope="session")
def small_cases():
    return load_small_cases()


@pytest.fixture(scope="session")
def digests():
    return json.loads((GOLDEN / "golden_digests.json").read_text())


def rings_equal(a, b) -> bool:
    return len(a) == len(b) and all(x.shape == y.shape and np.array_equal(x, y) for x, y in zip(a, b))


@pytest.fixture(scope="session")
def clipper():
    import sbclip
    c = sbclip.Clipper(0)
    yield c
    c.close()


def digest(*arrays) -> str:
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def ring_digest(rings) -> str:
    off = np.cumsum([0] + [len(r) for r in rings]).astype(np.int64)
    xy = np.concatenate(rings).astype(np.float64) if rings else np.zeros((0, 2))
    return digest(off, xy)


# One hand-made known-answer pair per classification type of the reference's
# lineSegmentIntersection (p_seg_tree/oacc_segment_tree.cpp:5408-5419):
# (p1, p2, q1, q2, expected type).
KAT_PAIRS = [
    ((0, 0), (2, 0), (5, 1), (5, 3), 0),        # disjoint
    ((0, 0), (2, 2), (0, 2), (2, 0), 1),        # X: proper crossing
    ((1, 0), (1, 3), (0, 0), (2, 0), 2),        # T on Q: P1 inside Q
    ((0, 0), (2, 0), (1, 0), (1, 3), 3),        # T on P: Q1 inside P
    ((0, 0), (2, 0), (0, 0), (0, 2), 4),        # V: shared start vertex
    ((0, 0), (4, 0), (1, 0), (-3, 0), 5),       # X overlap: Q1 in P and P1 in Q
    ((2, 0), (6, 0), (0, 0), (4, 0), 6),        # T overlap on Q
    ((0, 0), (6, 0), (2, 0), (9, 0), 7),        # T overlap on P
    ((0, 0), (2, 0), (0, 0), (3, 0), 8),        # V overlap
    ((0, 0), (1, 0), (0, 1), (1, 1), 0),        # parallel, not collinear
]


def load_union_cases():
    """Union fixtures: (kind, base, overlay, rings) from the reference's back end
    with its UNION switch set (tests/golden/make_golden.py)."""
    z = np.load(GOLDEN / "golden_union.npz")
    out, ro, ri = [], 0, 0
    for i, kind in enumerate(z["kind"]):
        b = z["b_xy"][z["b_off"][i]:z["b_off"][i + 1]]
        c = z["c_xy"][z["c_off"][i]:z["c_off"][i + 1]]
        rings = []
        for _ in range(int(z["r_ring_cnt"][i])):
            rings.append(z["r_xy"][z["r_off"][ro]:z["r_off"][ro + 1]])
            ro += 1
        out.append((str(kind), b, c, rings))
    return out


def load_component_cases():
    """[(kind, union, base components, overlay components, Foster's rings)]
    from golden_components.npz."""
    z = np.load(GOLDEN / "golden_components.npz")
    cases = []
    bv = cv = bi = ci = ro = 0
    for i, kind in enumerate(z["kind"]):
        comps = []
        for xy, cnt, n, pos in ((z["b_xy"], z["b_comp"], int(z["b_ncomp"][i]), "b"),
                                (z["c_xy"], z["c_comp"], int(z["c_ncomp"][i]), "c")):
            side = []
            for _ in range(n):
                if pos == "b":
                    m = int(cnt[bi]); side.append(xy[bv:bv + m]); bv += m; bi += 1
                else:
                    m = int(cnt[ci]); side.append(xy[cv:cv + m]); cv += m; ci += 1
            comps.append(side)
        rings = []
        for _ in range(int(z["r_ring_cnt"][i])):
            rings.append(z["r_xy"][z["r_off"][ro]:z["r_off"][ro + 1]])
            ro += 1
        cases.append((str(kind), bool(z["union"][i]), comps[0], comps[1], rings))
    return cases


def text6(rings):
    """Rings as Foster's program prints them (6 significant digits)."""
    return [[f"{x:.6g} {y:.6g}" for x, y in np.asarray(r, np.float64).reshape(-1, 2)]
            for r in rings]
