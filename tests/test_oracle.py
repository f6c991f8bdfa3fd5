"""CPU tests of the oracle (the C restatement) against the reference's own
outputs: golden fixtures made by the reference build, known-answer pairs,
and (when it is built here) the reference binary itself."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_py as O
import sbclip_gen as gen
from conftest import KAT_PAIRS, digest, ring_digest, rings_equal


@pytest.mark.parametrize("p1,p2,q1,q2,want", KAT_PAIRS)
def test_classifier_known_answers(p1, p2, q1, q2, want):
    t, _, _ = O.segment_intersection(p1, p2, q1, q2)
    assert t == want


def test_oracle_matches_reference_small_cases(small_cases):
    assert len(small_cases) >= 90
    for case in small_cases:
        res = O.clip(case.base, case.overlays)
        for i, ov in enumerate(res["overlays"]):
            assert rings_equal(O.rings_of(ov), case.rings[i]), case.kind
            ub, uc, ut = case.uniq[i]
            assert np.array_equal(ov["uniq_b"], ub) and np.array_equal(ov["uniq_c"], uc)
            assert np.array_equal(ov["uniq_t"], ut)


def _check_digests(entry, b, c):
    assert digest(b, c) == entry["input_sha256"], "generator output changed on this host"
    res = O.clip(b, [c])
    ov = res["overlays"][0]
    assert len(ov["raw_b"]) == entry["raw_hits"]
    assert len(ov["uniq_b"]) == entry["unique"]
    for arr in ("uniq_b", "uniq_c", "uniq_t", "isect_ab", "isect_ac", "merged_balpha",
                "merged_calpha", "merged_bnb", "merged_cnb", "label_b", "label_c"):
        assert digest(ov[arr].astype(np.int32)) == entry[arr + "_sha256"], arr
    for arr in ("isect_xy", "merged_bxy", "merged_cxy"):
        assert digest(ov[arr].astype(np.float64)) == entry[arr + "_sha256"], arr
    rings = O.rings_of(ov)
    assert len(rings) == entry["rings"]
    assert ring_digest(rings) == entry["rings_sha256"]


def test_oracle_matches_reference_10k_8k(digests):
    b, c = gen.pair_small()
    _check_digests(digests["pair_10k_8k"], b, c)


@pytest.mark.slow
def test_oracle_matches_reference_1m_1m(digests):
    b, c = gen.pair_large()
    _check_digests(digests["pair_1m_1m"], b, c)


@pytest.mark.skipif(not O.ref_available(), reason="reference binary not built here")
def test_oracle_matches_reference_binary_random_seeds():
    rng = np.random.default_rng(99)
    for t in range(6):
        nb = int(rng.integers(200, 800))
        nc = int(rng.integers(50, nb))
        b = gen.star(nb, 7000 + t)
        c = gen.star(nc, 8000 + t, centre=tuple(rng.uniform(-0.4, 0.4, 2)))
        try:
            ref = O.run_reference(b, [c], timeout=60)
        except RuntimeError:
            continue  # the reference build corrupts its heap on some inputs
        got = O.rings_of(O.clip(b, [c])["overlays"][0])
        assert rings_equal(got, ref["rings"][0])


def test_oracle_rejects_degenerate_polygons():
    with pytest.raises(O.OracleError):
        O.clip(np.array([[0, 0], [1, 0]], float), [gen.star(5, 1)])
