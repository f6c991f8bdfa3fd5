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


def _keys(xy):
    """Exact (x, y) keys as 16-byte records (-0.0 folded into 0.0, as Python
    float equality, and so the dict look-ups above, treat them)."""
    a = np.ascontiguousarray(np.asarray(xy, np.float64).reshape(-1, 2) + 0.0)
    return a.view(np.dtype((np.void, 16))).ravel()


def _first_index(table_xy, query_xy):
    """For every query point, the lowest index of an equal table point, or -1."""
    tk = _keys(table_xy)
    qk = _keys(query_xy)
    uk, first = np.unique(tk, return_index=True)
    pos = np.searchsorted(uk, qk)
    pos_c = np.minimum(pos, max(len(uk) - 1, 0))
    hit = (pos < len(uk)) & (uk[pos_c] == qk) if len(uk) else np.zeros(len(qk), bool)
    return np.where(hit, first[pos_c] if len(uk) else -1, -1)


def gradient_of_rings(base, overlay, rings, uniq_b, uniq_c, uniq_t, isect_xy):
    """(area, d area / d base, d area / d overlay) of given result rings with
    the provenance rules of area_gradient, vectorised with numpy (the same
    numbers: every product and sum is the same FP64 operation, only the
    order of the per-vertex accumulations may differ)."""
    b = np.ascontiguousarray(base, np.float64).reshape(-1, 2)
    c = np.ascontiguousarray(overlay, np.float64).reshape(-1, 2)
    nb, nc = len(b), len(c)
    gb = np.zeros((nb, 2))
    gc = np.zeros((nc, 2))
    if not rings:
        return 0.0, gb, gc
    R = np.concatenate(rings).reshape(-1, 2)
    lens = np.array([len(r) for r in rings])
    start = np.repeat(np.cumsum(lens) - lens, lens)
    pos = np.arange(len(R)) - start
    ln = np.repeat(lens, lens)
    nxt = start + (pos + 1) % ln
    prv = start + (pos - 1) % ln
    g = np.stack([0.5 * (R[nxt, 1] - R[prv, 1]), 0.5 * (R[prv, 0] - R[nxt, 0])], axis=1)
    ib = _first_index(b, R)
    ic = np.where(ib < 0, _first_index(c, R), -1)
    t1 = np.asarray(uniq_t) == 1
    ixy = np.asarray(isect_xy, np.float64).reshape(-1, 2)[t1]
    xb = np.asarray(uniq_b)[t1] // 2
    xc = np.asarray(uniq_c)[t1] // 2
    ix = np.where((ib < 0) & (ic < 0), _first_index(ixy, R), -1)
    if ((ib < 0) & (ic < 0) & (ix < 0)).any():
        k = int(np.flatnonzero((ib < 0) & (ic < 0) & (ix < 0))[0])
        raise ValueError(f"ring vertex {tuple(R[k])} has no provenance")
    m = ib >= 0
    np.add.at(gb, ib[m], g[m])
    m = ic >= 0
    np.add.at(gc, ic[m], g[m])
    m = ix >= 0
    if m.any():
        gg = g[m]
        i1, j1 = xb[ix[m]], xc[ix[m]]
        i2, j2 = (i1 + 1) % nb, (j1 + 1) % nc
        b1, b2, c1, c2 = b[i1], b[i2], c[j1], c[j2]

        def area3(p, q, r):
            A = (q[:, 0] - p[:, 0]) * (r[:, 1] - p[:, 1]) - (q[:, 1] - p[:, 1]) * (r[:, 0] - p[:, 0])
            dP = np.stack([q[:, 1] - r[:, 1], r[:, 0] - q[:, 0]], 1)
            dQ = np.stack([r[:, 1] - p[:, 1], p[:, 0] - r[:, 0]], 1)
            dR = np.stack([p[:, 1] - q[:, 1], q[:, 0] - p[:, 0]], 1)
            return A, dP, dQ, dR

        A1, dP1, dQ1, dR1 = area3(b1, c1, c2)
        A2, dP2, dQ2, dR2 = area3(b2, c1, c2)
        d = A1 - A2
        al = A1 / d
        ga = np.einsum("ij,ij->i", gg, b2 - b1)
        k1 = -A2 / (d * d) * ga
        k2 = A1 / (d * d) * ga
        np.add.at(gb, i1, (1.0 - al)[:, None] * gg + k1[:, None] * dP1)
        np.add.at(gb, i2, al[:, None] * gg + k2[:, None] * dP2)
        np.add.at(gc, j1, k1[:, None] * dQ1 + k2[:, None] * dQ2)
        np.add.at(gc, j2, k1[:, None] * dR1 + k2[:, None] * dR2)
    return shoelace(rings), gb, gc


def area_gradient_fast(base, overlay):
    """area_gradient with the vectorised provenance and chain rule."""
    ov = O.clip(base, [overlay])["overlays"][0]
    return gradient_of_rings(base, overlay, O.rings_of(ov), ov["uniq_b"], ov["uniq_c"],
                             ov["uniq_t"], ov["isect_xy"])


def _two_prod(a, b):
    """p = fl(a*b) and the exact error e = a*b - p (Dekker's product with
    Veltkamp's split; no FMA, no overflow for |a|, |b| < 2^996)."""
    p = a * b
    t = 134217729.0 * a
    ah = t - (t - a)
    al = a - ah
    t = 134217729.0 * b
    bh = t - (t - b)
    bl = b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def exact_shoelace(rings) -> float:
    """Shoelace area of the rings with every cross product and the sum taken
    exactly, rounded once (finite differences of it are free of the FP64
    summation noise that a plain shoelace sum of a long ring carries)."""
    import math

    parts = []
    for r in rings:
        r = np.asarray(r, np.float64)
        x, y = r[:, 0], r[:, 1]
        xn, yn = np.roll(x, -1), np.roll(y, -1)
        p1, e1 = _two_prod(x, yn)
        p2, e2 = _two_prod(xn, y)
        parts += [p1, e1, -p2, -e2]
    if not parts:
        return 0.0
    return 0.5 * math.fsum(np.concatenate(parts).tolist())
