"""The classifier's early exit (seg_isect<true> in csrc/sbc_internal.cuh) on the
CPU: wherever its quotient bounds say that alpha or beta rounds outside
[-eps, 1 - eps), the oracle's lineSegmentIntersection (oacc_segment_tree.cpp:
5426-5517) must return type 0.  The areas are formed as area3 forms them
(IEEE double, round to nearest, no fused multiply-add), so the numpy values
are the kernel's values."""
from __future__ import annotations

import numpy as np

import oracle_py as O

EPS = 1e-9


def area3(px, py, qx, qy, rx, ry):
    return (qx - px) * (ry - py) - (qy - py) * (rx - px)


def quot_outside(n, d):
    m = (-4.0 * EPS) * d
    return np.where(d > 0.0, (n > 2.0 * d) | (n < m), (d < 0.0) & ((n < 2.0 * d) | (n > m)))


def early_exit(p1, p2, q1, q2):
    ap1 = area3(p1[:, 0], p1[:, 1], q1[:, 0], q1[:, 1], q2[:, 0], q2[:, 1])
    ap2 = area3(p2[:, 0], p2[:, 1], q1[:, 0], q1[:, 1], q2[:, 0], q2[:, 1])
    d = ap1 - ap2
    aq1 = area3(q1[:, 0], q1[:, 1], p1[:, 0], p1[:, 1], p2[:, 0], p2[:, 1])
    aq2 = area3(q2[:, 0], q2[:, 1], p1[:, 0], p1[:, 1], p2[:, 0], p2[:, 1])
    e = aq1 - aq2
    branch = np.abs(d) > EPS
    return branch & (quot_outside(ap1, d) | quot_outside(aq1, e))


def _pairs(rng, n):
    """Random pairs, pairs whose endpoints sit on or next to the other segment,
    parallel and collinear pairs, at several scales."""
    out = []
    for scale in (1e-6, 1.0, 1e3, 1e6):
        p1 = rng.uniform(-1, 1, (n, 2)) * scale
        p2 = p1 + rng.normal(0, 0.3, (n, 2)) * scale
        q1 = rng.uniform(-1, 1, (n, 2)) * scale
        q2 = q1 + rng.normal(0, 0.3, (n, 2)) * scale
        out.append((p1, p2, q1, q2))
        # q1 at alpha in {0, 1, just outside, just inside} of p's segment
        t = rng.choice([0.0, 1.0, -1e-9, 1e-9, 1 - 1e-9, 1 + 1e-9, 2.0, -4e-9, 2 + 1e-15], (n, 1))
        q1b = p1 + t * (p2 - p1) + rng.normal(0, 1e-12, (n, 2)) * scale
        out.append((p1, p2, q1b, q2))
        # parallel and collinear
        off = rng.choice([0.0, 1e-12, 1e-3], (n, 1)) * scale
        q1c = p1 + rng.uniform(-1, 2, (n, 1)) * (p2 - p1) + off
        q2c = q1c + rng.uniform(-1, 1, (n, 1)) * (p2 - p1)
        out.append((p1, p2, q1c, q2c))
    return [np.concatenate(x) for x in zip(*out)]


def test_early_exit_only_where_the_classifier_returns_zero():
    rng = np.random.default_rng(8800)
    p1, p2, q1, q2 = _pairs(rng, 1500)
    ex = early_exit(p1, p2, q1, q2)
    assert ex.sum() > len(ex) // 4  # the exit is taken often
    bad = []
    for i in np.flatnonzero(ex):
        t, _, _ = O.segment_intersection(p1[i], p2[i], q1[i], q2[i])
        if t != 0:
            bad.append(i)
    assert not bad, bad[:5]
    # and pairs the classifier keeps are never cut short
    kept = [i for i in np.flatnonzero(~ex)[:2000]]
    assert any(O.segment_intersection(p1[i], p2[i], q1[i], q2[i])[0] != 0 for i in kept)
