"""GPU parity of union mode (SBC_FLAG_UNION) against the reference's own
back end with its UNION switch set: the pair pipeline, the batched engine
and the one-base-many-overlays engine, rings bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import sbclip_gen as gen
from conftest import load_union_cases, rings_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def uc():
    import sbclip
    c = sbclip.Clipper(0, union=True)
    yield c
    c.close()


def test_union_pair_matches_reference(uc):
    for kind, b, c, want in load_union_cases():
        assert rings_equal(uc.clip_pair(b, c), want), kind


def test_union_batch_matches_reference(uc):
    cases = load_union_cases()
    rings, st = uc.clip_batch([x[1] for x in cases], [x[2] for x in cases])
    assert (st == 0).all()
    for (kind, b, c, want), got in zip(cases, rings):
        assert rings_equal(got, want), kind


def test_union_pairwise_matches_pair_path(uc):
    base, ovs = gen.one_to_many(n_base=4_000, n_overlays=60, seed=3400, hi=800,
                                near_boundary=0.6)
    got, st = uc.clip_pairwise(base, ovs)
    assert (st == 0).all()
    for i, c in enumerate(ovs):
        assert rings_equal(got[i], uc.clip_pair(base, c)), i
    # the split path (records through the pipeline's rows) in union mode too
    uc.set_pairwise_split(1)
    try:
        got2, _ = uc.clip_pairwise(base, ovs)
    finally:
        uc.set_pairwise_split(8192)
    assert all(rings_equal(a, b) for a, b in zip(got, got2))


def test_union_pairwise_touching_overlays(uc):
    """Overlays touching the base exactly (see the intersection version in
    test_gpu_pairwise.py) in union mode: the pairwise engine against the pair
    path, rings and statuses."""
    import sbclip
    base = np.array([[0.0, -8.0], [6.0, -6.0], [8.0, 0.0], [6.0, 6.0], [0.0, 8.0],
                     [-6.0, 6.0], [-8.0, 0.0], [-6.0, -6.0]])
    on1 = lambda x: [x, -8.0 + x / 3.0]
    on2 = lambda x: [x, -6.0 + 3.0 * (x - 6.0)]
    ovs = [
        np.array([[2.0, -9.0], on1(3.0), [4.0, -9.5]]),
        np.array([[2.0, -5.0], [4.0, -5.5], on1(3.0)]),
        np.array([on1(1.5), on1(4.5), [4.5, -4.0], [1.5, -5.0]]),
        np.array([on1(1.5), on1(4.5), [4.5, -9.0], [1.5, -9.5]]),
        np.array([on1(3.0), [7.5, -7.5], on2(7.0)]),
        np.array([on1(3.0), on2(7.0), [4.5, -3.0]]),
    ]
    got, st = uc.clip_pairwise(base, ovs)
    for i, c in enumerate(ovs):
        try:
            want = uc.clip_pair(base, c)
        except sbclip.SbcError as e:
            assert st[i] == e.code, (i, st[i], e.code)
            continue
        assert st[i] == 0, (i, st[i])
        assert rings_equal(got[i], want), i
