#!/usr/bin/env python3
"""Regenerate the golden fixtures from the reference's own CPU build.

    python oracle/build_ref.py && python tests/golden/make_golden.py
    (--union-only / --components-only: just that fixture)

Outputs (committed):
  golden_small.npz   ~100 small cases (random stars, integer-grid polygons
                     with T/V/overlap degeneracies, axis-aligned rectangles,
                     one-to-many runs): inputs and the reference's rings at
                     full precision, plus its unique candidate pairs.
  golden_components.npz  multi-component polygons (holes and islands, the
                     .poly format of lib/optimizedFostersAlgorithm): inputs and
                     the rings of the reference's Foster program (precision 6,
                     its output format), intersection and union.  The seg
                     driver takes one ring per file; Foster's program is the
                     reference's own code for several components.  Generic
                     positions, plus components identical to the other side's
                     (the identical-component rule): on partly shared edges
                     the seg path and Foster's program differ already for
                     single rings, so those are not fixtures.
  golden_digests.json  SHA-256 digests of the reference's rings and
                     intermediate arrays for the 10k x 8k star pair and the
                     1M x 1M jagged pair (inputs regenerated from their seeds).

Cases on which the reference build crashes or loops (heap corruption from its
reads past array ends) are not fixtures: the reference defines no output
there.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "segment-tree-based-clipping_gb300"))
import oracle_py as O  # noqa: E402
import sbclip_gen as gen  # noqa: E402

OUT = Path(__file__).resolve().parent


def grid_star(n, seed, c=(0, 0)):
    r = np.random.default_rng(seed)
    th = np.sort(r.choice(np.arange(64), n, replace=False)) / 64.0 * 2.0 * np.pi
    rad = r.integers(2, 6, n)
    sn, cs = gen.sincos(th)
    xy = np.stack([np.round(c[0] + rad * cs), np.round(c[1] + rad * sn)], 1)
    keep = np.ones(len(xy), bool)
    keep[1:] = np.any(xy[1:] != xy[:-1], 1)
    xy = xy[keep]
    if len(xy) > 1 and np.all(xy[0] == xy[-1]):
        xy = xy[:-1]
    return xy


def small_cases():
    rng = np.random.default_rng(20261203)
    cases = []
    for t in range(40):
        nb = int(rng.integers(4, 80))
        nc = int(rng.integers(3, nb + 1))
        cases.append(("star", gen.star(nb, 100 + t),
                      [gen.star(nc, 200 + t, centre=tuple(rng.uniform(-0.5, 0.5, 2)))]))
    for t in range(40):
        b = grid_star(int(rng.integers(5, 24)), 300 + t)
        c = grid_star(int(rng.integers(4, 24)), 400 + t, c=tuple(rng.integers(-2, 3, 2)))
        if len(c) > len(b):
            b, c = c, b
        if len(b) >= 3 and len(c) >= 3:
            cases.append(("grid", b, [c]))
    for t in range(16):
        x0, y0 = rng.integers(-3, 3, 2)
        w, h = rng.integers(1, 5, 2)
        b = np.array([[0, 0], [4, 0], [4, 4], [0, 4]], float)
        c = np.array([[x0, y0], [x0 + w, y0], [x0 + w, y0 + h], [x0, y0 + h]], float)
        cases.append(("rect", b, [c]))
    for t in range(8):
        k = int(rng.integers(2, 4))
        b = gen.star(int(rng.integers(60, 120)), 500 + t)
        ovs = [gen.star(int(rng.integers(3, 50)), 600 + 10 * t + i,
                        centre=tuple(rng.uniform(-0.6, 0.6, 2))) for i in range(k)]
        cases.append(("multi", b, ovs))
    # fixed shapes: disjoint, contained, identical, nested squares
    sq = np.array([[0, 0], [4, 0], [4, 4], [0, 4]], float)
    cases.append(("fixed", gen.star(30, 1), [gen.star(12, 2, centre=(5.0, 5.0))]))
    cases.append(("fixed", gen.star(30, 1), [gen.star(12, 2, centre=(0.0, 0.0), R=0.1)]))
    cases.append(("fixed", sq, [sq.copy()]))
    cases.append(("fixed", sq, [np.array([[1, 1], [2, 1], [2, 2], [1, 2]], float)]))
    return cases


def digest(*arrays) -> str:
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


def text6(rings) -> str:
    out = []
    for r in rings:
        out.append(",\n".join(f"{x:.6g} {y:.6g}" for x, y in r) + ";\n")
    return "".join(out)


def main():
    if not O.ref_available():
        raise SystemExit("build the reference first: python oracle/build_ref.py")
    # ---- small cases
    store = {"kind": [], "b_off": [0], "b_xy": [], "c_off": [0], "c_cnt": [], "c_xy": [],
             "r_ring_cnt": [], "r_off": [0], "r_xy": [], "u_off": [0], "u_b": [], "u_c": [], "u_t": []}
    n_ok = n_skip = 0
    for kind, b, ovs in small_cases():
        try:
            res = O.run_reference(b, ovs, dump=True, timeout=30)
        except Exception:
            n_skip += 1
            continue
        n_ok += 1
        store["kind"].append(kind)
        store["b_xy"].append(b)
        store["b_off"].append(store["b_off"][-1] + len(b))
        store["c_cnt"].append(len(ovs))
        for o in ovs:
            store["c_xy"].append(o)
            store["c_off"].append(store["c_off"][-1] + len(o))
        for i, rings in enumerate(res["rings"]):
            store["r_ring_cnt"].append(len(rings))
            for r in rings:
                store["r_xy"].append(r)
                store["r_off"].append(store["r_off"][-1] + len(r))
            d = res["dumps"][i + 1]
            store["u_b"].append(d.get("uniq_b", np.zeros(0, np.int64)))
            store["u_c"].append(d.get("uniq_c", np.zeros(0, np.int64)))
            store["u_t"].append(d.get("uniq_t", np.zeros(0, np.int64)))
            store["u_off"].append(store["u_off"][-1] + len(store["u_b"][-1]))
    cat = lambda xs, dt: (np.concatenate([np.asarray(x, dt).reshape(-1, *np.asarray(x).shape[1:]) for x in xs])
                          if xs else np.zeros(0, dt))
    np.savez_compressed(
        OUT / "golden_small.npz",
        kind=np.array(store["kind"]),
        b_off=np.array(store["b_off"], np.int64), b_xy=np.concatenate(store["b_xy"]).astype(np.float64),
        c_off=np.array(store["c_off"], np.int64), c_cnt=np.array(store["c_cnt"], np.int64),
        c_xy=np.concatenate(store["c_xy"]).astype(np.float64),
        r_ring_cnt=np.array(store["r_ring_cnt"], np.int64), r_off=np.array(store["r_off"], np.int64),
        r_xy=(np.concatenate(store["r_xy"]).astype(np.float64) if store["r_xy"] else np.zeros((0, 2))),
        u_off=np.array(store["u_off"], np.int64),
        u_b=cat(store["u_b"], np.int64), u_c=cat(store["u_c"], np.int64), u_t=cat(store["u_t"], np.int64),
    )
    print(f"small cases: {n_ok} stored, {n_skip} skipped (reference crashed)")

    # ---- large configurations
    dig = {}
    for name, make, threads in (("pair_10k_8k", gen.pair_small, 1), ("pair_1m_1m", gen.pair_large, 1)):
        b, c = make()
        res = O.run_reference(b, [c], threads=threads, dump=True, timeout=3000)
        rings = res["rings"][0]
        d = res["dumps"][1]
        entry = {
            "input_sha256": digest(b, c),
            "nb": int(len(b)), "nc": int(len(c)),
            "raw_hits": int(len(d["raw_b"])), "unique": int(len(d["uniq_b"])),
            "rings": len(rings), "vertices": int(sum(len(r) for r in rings)),
            "rings_sha256": ring_digest(rings),
            "text6_sha256": hashlib.sha256(text6(rings).encode()).hexdigest(),
            "reference_time_line_us": res["time_line"], "reference_threads": threads,
        }
        for arr in ("uniq_b", "uniq_c", "uniq_t", "isect_ab", "isect_ac", "merged_balpha",
                    "merged_calpha", "merged_bnb", "merged_cnb", "label_b", "label_c"):
            entry[arr + "_sha256"] = digest(d[arr].astype(np.int32))
        for arr in ("isect_xy", "merged_bxy", "merged_cxy"):
            entry[arr + "_sha256"] = digest(d[arr].astype(np.float64))
        dig[name] = entry
        print(name, {k: v for k, v in entry.items() if not k.endswith("sha256")})
    (OUT / "golden_digests.json").write_text(json.dumps(dig, indent=1) + "\n")


def main_union():
    """Union fixtures: the reference's Foster back end with its UNION switch
    set (the harness's SBC_REF_UNION), one overlay per case: the small cases
    with a single overlay, plus two star pairs of a few thousand vertices."""
    if not O.ref_available():
        raise SystemExit("build the reference first: python oracle/build_ref.py")
    cases = [(k, b, ovs[0]) for k, b, ovs in small_cases() if len(ovs) == 1]
    cases.append(("stars-3000-2500", gen.star(3000, 71), gen.star(2500, 72, centre=(0.2, -0.1))))
    cases.append(("stars-1200-900", gen.star(1200, 73), gen.star(900, 74, centre=(-0.3, 0.25))))
    store = {"kind": [], "b_off": [0], "b_xy": [], "c_off": [0], "c_xy": [], "r_ring_cnt": [],
             "r_off": [0], "r_xy": []}
    n_ok = n_skip = 0
    for kind, b, c in cases:
        try:
            res = O.run_reference(b, [c], timeout=30, union=True)
        except Exception:
            n_skip += 1
            continue
        n_ok += 1
        store["kind"].append(kind)
        store["b_xy"].append(b)
        store["b_off"].append(store["b_off"][-1] + len(b))
        store["c_xy"].append(c)
        store["c_off"].append(store["c_off"][-1] + len(c))
        rings = res["rings"][0]
        store["r_ring_cnt"].append(len(rings))
        for r in rings:
            store["r_xy"].append(r)
            store["r_off"].append(store["r_off"][-1] + len(r))
    np.savez_compressed(
        OUT / "golden_union.npz",
        kind=np.array(store["kind"]),
        b_off=np.array(store["b_off"], np.int64), b_xy=np.concatenate(store["b_xy"]).astype(np.float64),
        c_off=np.array(store["c_off"], np.int64), c_xy=np.concatenate(store["c_xy"]).astype(np.float64),
        r_ring_cnt=np.array(store["r_ring_cnt"], np.int64), r_off=np.array(store["r_off"], np.int64),
        r_xy=(np.concatenate(store["r_xy"]).astype(np.float64) if store["r_xy"] else np.zeros((0, 2))),
    )
    print(f"union cases: {n_ok} stored, {n_skip} skipped (reference crashed)")


def component_cases():
    cases = []
    for t in range(24):
        n1 = [16, 40, 200, 600][t % 4]
        n2 = [16, 30, 300, 500][(t // 4) % 4]
        hb, hc = t % 3 + 1, (t // 3) % 4
        b = gen.holed(n1, 600 + t, R=1.0, holes=hb, islands=min(t % 2, hb))
        c = gen.holed(n2, 700 + t, centre=(0.3 * np.cos(t), 0.3 * np.sin(t)), R=0.9, holes=hc,
                      islands=min((t // 5) % 2, hc))
        cases.append(("generic", b, c))
    for t in range(4):
        b = gen.holed(60 + 20 * t, 800 + t, R=1.0, holes=2, islands=1)
        cases.append(("identical", b, [x.copy() for x in b]))
        cases.append(("identical outer", b, [b[0]]))
        cases.append(("hole as outer", b, [b[1][::-1].copy()]))
    return cases


def main_components():
    if not O.foster_available():
        raise SystemExit("build the reference first: python oracle/build_ref.py")
    store = {"kind": [], "union": [], "b_xy": [], "b_comp": [], "b_ncomp": [], "c_xy": [],
             "c_comp": [], "c_ncomp": [], "r_ring_cnt": [], "r_off": [0], "r_xy": []}
    for kind, b, c in component_cases():
        for union in (False, True):
            rings = O.run_foster(b, c, timeout=60, union=union)["rings"]
            store["kind"].append(kind)
            store["union"].append(union)
            for side, comps in (("b", b), ("c", c)):
                store[side + "_xy"].extend(comps)
                store[side + "_comp"].extend(len(x) for x in comps)
                store[side + "_ncomp"].append(len(comps))
            store["r_ring_cnt"].append(len(rings))
            for r in rings:
                store["r_xy"].append(r)
                store["r_off"].append(store["r_off"][-1] + len(r))
    np.savez_compressed(
        OUT / "golden_components.npz",
        kind=np.array(store["kind"]), union=np.array(store["union"], bool),
        b_xy=np.concatenate(store["b_xy"]).astype(np.float64),
        b_comp=np.array(store["b_comp"], np.int64), b_ncomp=np.array(store["b_ncomp"], np.int64),
        c_xy=np.concatenate(store["c_xy"]).astype(np.float64),
        c_comp=np.array(store["c_comp"], np.int64), c_ncomp=np.array(store["c_ncomp"], np.int64),
        r_ring_cnt=np.array(store["r_ring_cnt"], np.int64), r_off=np.array(store["r_off"], np.int64),
        r_xy=(np.concatenate(store["r_xy"]).astype(np.float64) if store["r_xy"] else np.zeros((0, 2))),
    )
    print(f"component cases: {len(store['kind'])} stored")


if __name__ == "__main__":
    import sys as _sys
    if "--union-only" in _sys.argv:
        main_union()
    elif "--components-only" in _sys.argv:
        main_components()
    else:
        main()
        main_union()
        main_components()
