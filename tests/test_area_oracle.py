"""CPU checks of the differentiation oracle (oracle/area_grad.py): the FP64
area gradient built from the reference-equivalent rings agrees with central
finite differences of the area (h = 1e-7) to 1e-8 relative."""
from __future__ import annotations

import numpy as np

import area_grad as AG
import sbclip_gen as gen


def test_host_gradient_matches_finite_differences():
    for b, c in gen.small_pairs(5, seed=91, lo=4, hi=24):
        A, gb, gc = AG.area_gradient(b, c)
        fb, fc = AG.finite_difference(b, c)
        an = np.concatenate([gb.ravel(), gc.ravel()])
        fd = np.concatenate([fb.ravel(), fc.ravel()])
        scale = max(np.abs(an).max(), abs(A), 1e-300)
        assert np.abs(an - fd).max() <= 1e-8 * scale


def test_area_is_the_shoelace_of_the_rings():
    b, c = gen.star(40, 3), gen.star(30, 4, centre=(0.2, -0.1))
    A, _, _ = AG.area_gradient(b, c)
    assert A == AG.area(b, c)
    assert abs(A) > 0.1


def test_vectorised_gradient_equals_loop_gradient():
    for b, c in gen.small_pairs(40, seed=77):
        a1, gb1, gc1 = AG.area_gradient(b, c)
        a2, gb2, gc2 = AG.area_gradient_fast(b, c)
        s = max(np.abs(gb1).max(), np.abs(gc1).max(), 1e-300)
        assert a1 == a2
        assert np.abs(gb1 - gb2).max() <= 1e-14 * s and np.abs(gc1 - gc2).max() <= 1e-14 * s


def test_exact_shoelace_is_exact():
    from fractions import Fraction
    rng = np.random.default_rng(3)
    for _ in range(20):
        rings = [rng.uniform(-1e3, 1e3, (int(rng.integers(3, 40)), 2)) for _ in range(2)]
        ex = Fraction(0)
        for q in rings:
            for i in range(len(q)):
                j = (i + 1) % len(q)
                ex += Fraction(q[i, 0]) * Fraction(q[j, 1]) - Fraction(q[j, 0]) * Fraction(q[i, 1])
        assert AG.exact_shoelace(rings) == float(ex / 2)


def test_parallel_oracle_runs_equal_serial_runs():
    import oracle_py as O
    from conftest import rings_equal
    pairs = gen.small_pairs(24, seed=91)
    par = O.clip_pairs_parallel(pairs, threads=4)
    for (b, c), (st, rings) in zip(pairs, par):
        assert st == 0
        assert rings_equal(rings, O.rings_of(O.clip(b, [c])["overlays"][0]))


def test_oracle_tree_arrays_are_consistent():
    import oracle_py as O
    b, c = gen.pair_small()
    run = O.clip(b, [c])
    t, s = run["tree"], run["stats"]
    assert len(t["ea"]) == s["elem_count"] and np.all(np.diff(t["ea"]) >= 0)
    assert t["leaf_off"][-1] == s["leaf_end_total"] == len(t["leaf_edge"])
    assert t["cov_off"][-1] == s["cover_total"] == len(t["cov_edge"])
    assert len(t["cov_off"]) == s["tree_size"] + 1
