"""Intersection area and its gradient from the oracle's rings.

TEST INFRASTRUCTURE ONLY: the checker of the batched area forward/backward
entry points, never the product.

The reference computes no areas or gradients.  The area of a clipping result
is the FP64 shoelace sum over its rings (the reference's output rings,
foster/polyclip.h:861-869).  Its gradient with the combinatorial structure
held fixed follows from where each ring vertex comes from:

* a base or an overlay vertex: its gradient goes to that vertex;
* a proper crossing (type 1 of lineSegmentIntersection2,
  p_seg_tree/oacc_segment_tree.cpp:5520-5611) of base edge b1b2 with overlay
  edge c1c2: I = (1 - a) b1 + a b2 (saveIntersectionsParallel, :7257-7341)
  with a = A(b1,c1,c2) / (A(b1,c1,c2) - A(b2,c1,c2)), chained through a.

Provenance is found by exact coordinate match (ring vertices are bit-exact
copies): base vertices first, then overlay vertices, then the crossings of
the unique intersection records.
"""
from __future__ import annotations

import numpy as np

import oracle_py as O


def shoelace(rings) -> float:
    a = 0.0
    for r in rings:
        x, y = r[:, 0], r[:, 1]
        a += 0.5 * float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))
    return a


def area(base, overlay) -> float:
    return shoelace(O.rings_of(O.clip(base, [overlay])["overlays"][0]))


def _area3_grads(p, q, r):
    """A(P,Q,R) = (Qx-Px)(Ry-Py) - (Qy-Py)(Rx-Px) and its partials."""
    A = (q[0] - p[0]) * (r[1] - p[1]) - (q[1] - p[1]) * (r[0] - p[0])
    dP = np.array([q[1] - r[1], r[0] - q[0]])
    dQ = np.array([r[1] - p[1], p[0] - r[0]])
    dR = np.array([p[1] - q[1], q[0] - p[0]])
    return A, dP, dQ, dR


def area_gradient(base, overlay):
    """(area, d area / d base (nb,2), d area / d overlay (nc,2))."""
    b = np.ascontiguousarray(base, np.float64).reshape(-1, 2)
    c = np.ascontiguousarray(overlay, np.float64).reshape(-1, 2)
    run = O.clip(b, [c])
    ov = run["overlays"][0]
    rings = O.rings_of(ov)
    nb, nc = len(b), len(c)
    bmap, cmap, xmap = {}, {}, {}
    for i in range(nb - 1, -1, -1):
        bmap[(b[i, 0], b[i, 1])] = i
    for j in range(nc - 1, -1, -1):
        cmap[(c[j, 0], c[j, 1])] = j
    ub, uc, ut, ixy = ov["uniq_b"], ov["uniq_c"], ov["uniq_t"], ov["isect_xy"].reshape(-1, 2)
    for k in range(len(ub) - 1, -1, -1):
        if ut[k] == 1:
            xmap[(ixy[k, 0], ixy[k, 1])] = (ub[k] // 2, uc[k] // 2)
    gb = np.zeros((nb, 2))
    gc = np.zeros((nc, 2))
    for r in rings:
        m = len(r)
        for i in range(m):
            x, y = r[i]
            xp, yp = r[(i + 1) % m]
            xm, ym = r[(i - 1) % m]
            g = np.array([0.5 * (yp - ym), 0.5 * (xm - xp)])
            key = (x, y)
            if key in bmap:
                gb[bmap[key]] += g
            elif key in cmap:
                gc[cmap[key]] += g
            elif key in xmap:
                i1, j1 = xmap[key]
                i2, j2 = (i1 + 1) % nb, (j1 + 1) % nc
                b1, b2, c1, c2 = b[i1], b[i2], c[j1], c[j2]
                A1, dP1, dQ1, dR1 = _area3_grads(b1, c1, c2)
                A2, dP2, dQ2, dR2 = _area3_grads(b2, c1, c2)
                d = A1 - A2
                al = A1 / d
                ga = float(g @ (b2 - b1))
                k1, k2 = -A2 / (d * d) * ga, A1 / (d * d) * ga
                gb[i1] += (1.0 - al) * g + k1 * dP1
                gb[i2] += al * g + k2 * dP2
                gc[j1] += k1 * dQ1 + k2 * dQ2
                gc[j2] += k1 * dR1 + k2 * dR2
            else:
                raise ValueError(f"ring vertex {key} has no provenance")
    return shoelace(rings), gb, gc


def finite_difference(base, overlay, h: float = 1e-7):
    """Central differences of the oracle's area in every coordinate."""
    b = np.array(base, np.float64).reshape(-1, 2)
    c = np.array(overlay, np.float64).reshape(-1, 2)
    gb = np.zeros_like(b)
    gc = np.zeros_like(c)
    for P, G in ((b, gb), (c, gc)):
        for i in range(P.shape[0]):
            for k in range(2):
                v = P[i, k]
                P[i, k] = v + h
                ap = area(b, c)
                P[i, k] = v - h
                am = area(b, c)
                P[i, k] = v
                G[i, k] = (ap - am) / (2 * h)
    return gb, gc
