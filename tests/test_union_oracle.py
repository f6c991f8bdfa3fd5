"""The oracle's union mode against the reference's own back end with its
UNION switch set (golden_union.npz): rings bit for bit."""
from __future__ import annotations

import oracle_py as O
from conftest import load_union_cases, rings_equal


def test_oracle_union_matches_reference_fixtures():
    cases = load_union_cases()
    assert len(cases) > 90
    for kind, b, c, want in cases:
        got = O.rings_of(O.clip(b, [c], union=True)["overlays"][0])
        assert rings_equal(got, want), kind


def test_union_differs_from_intersection():
    # the switch is live: a crossing pair's union is not its intersection
    kind, b, c, want = [x for x in load_union_cases() if x[0].startswith("stars-1200")][0]
    inter = O.rings_of(O.clip(b, [c])["overlays"][0])
    assert not rings_equal(inter, want)
