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
