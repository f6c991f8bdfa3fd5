"""Multi-component polygons (holes and islands) in the oracle, against the
reference's Foster program (golden_components.npz, its 6-digit output), and
the one-component case against the single-ring restatement."""
from __future__ import annotations

import numpy as np

import oracle_py as O
from conftest import load_component_cases, load_small_cases, rings_equal, text6


def test_oracle_components_match_foster_fixtures():
    cases = load_component_cases()
    assert len(cases) >= 72
    kinds = {k for k, *_ in cases}
    assert {"generic", "identical", "identical outer", "hole as outer"} <= kinds
    for kind, union, b, c, want in cases:
        got = O.rings_of(O.clip_components(b, c, union=union)["overlays"][0])
        assert text6(got) == text6(want), (kind, union)


def test_one_component_is_the_single_ring_restatement():
    n = 0
    for case in load_small_cases():
        if len(case.overlays) != 1:
            continue
        try:
            want = O.rings_of(O.clip(case.base, case.overlays)["overlays"][0])
        except O.OracleError as e:
            try:
                O.clip_components([case.base], case.overlays)
            except O.OracleError as e2:
                assert e2.status == e.status
                continue
            raise AssertionError("the components entry accepted what the single-ring one refused")
        got = O.rings_of(O.clip_components([case.base], case.overlays)["overlays"][0])
        assert rings_equal(got, want), case.kind
        n += 1
    assert n > 60


def test_component_offsets_are_checked():
    sq = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float64)
    tri = np.array([[5, 5], [6, 5], [5, 6]], np.float64)
    # a two-vertex component is refused
    try:
        O.clip_components([sq, tri[:2]], [sq + 0.5])
    except O.OracleError as e:
        assert e.status != 0
    else:
        raise AssertionError("two-vertex component accepted")
    # an overlay around one component only: that component comes back whole
    box = np.array([[4, 4], [7, 4], [7, 7], [4, 7]], np.float64)
    got = O.rings_of(O.clip_components([sq, tri], [box])["overlays"][0])
    assert len(got) == 1 and np.array_equal(got[0], tri)
