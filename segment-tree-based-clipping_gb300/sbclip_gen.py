"""Seeded synthetic star-shaped polygons for the segment-tree clipping workloads.

The reference's own datasets (real-world ocean / continent / lake / park rings)
are not available, so every workload is a seeded synthetic stand-in with the
shapes and sizes of the benchmark configurations:

* ``star``            vertex i at angle theta_i (n sorted, distinct U[0, 2pi)
                      draws), radius R*(0.5 + 0.5*u_i), counter-clockwise.
* ``jagged_star``     the same angles with radius R*(1 + 0.3*g_i), g the sum of
                      8 octaves of periodic 1-D value noise over theta (amplitude
                      halving per octave), clamped to >= 0.2R.
* ``pair_small``      10k x 8k plain stars (base at (0,0), overlay at (0.3,0.2)).
* ``pair_large``      1M x 1M jagged stars, R = 1000; overlay offset
                      (0.25R, 0.1R) and rotated 0.3 rad about its centre.
* ``uneven_pairs``    many independent pairs with vertex counts log-uniform in
                      [3, 2048] per polygon (plain stars, overlay centre offset
                      U[-0.5,0.5]^2; angles stratified: vertex k at
                      2pi (k + u_k) / n, so each polygon is simple without a
                      per-polygon sort), plus a few large jagged pairs (the
                      ``pair_large`` generator at 200k vertices) mixed in;
                      returned packed.
* ``holed``           one polygon as components (Foster's .poly layout): an
                      outer ring (stratified angles, radius R*U[0.7, 1]), holes
                      (radius R*U[0.12, 0.2], clockwise) on a circle of radius
                      0.35R, and islands (radius R*U[0.04, 0.08]) inside the
                      first holes; the bounds keep every component simple and
                      disjoint from the others.
* ``one_to_many``     one jagged base (200k vertices, R = 1000) against many
                      plain-star overlays: sizes log-uniform in [4, 5000], radii
                      log-uniform in [0.001R, 0.05R], centres uniform in the
                      base's bounding box (or, with ``near_boundary``, that
                      fraction of them on base vertices).

Files use the reference's text format (``src/clip.cpp:181-298``): the vertex
count on the first line, then one ``x,y`` line per vertex, no closing duplicate.
Seeds follow ``1000*config + polygon_index`` with NumPy's PCG64.
"""
from __future__ import annotations

import numpy as np

TWO_PI = 2.0 * np.pi

# Base lattice frequency (cells around the circle) of the lowest noise octave of
# the large jagged pair; chosen so that the 1M x 1M pair has 1e5..1e6 unique
# edge intersections.
JAGGED_BASE_FREQ = 6000


_HALF_PI_HI = float.fromhex("0x1.921fb544p+0")        # pi/2 to 33 bits (q*HI is exact)
_HALF_PI_LO = 1.5707963267948966 - _HALF_PI_HI
_SIN_C = [(-1) ** k / float(np.prod(np.arange(1, 2 * k + 2, dtype=np.float64))) for k in range(9)]
_COS_C = [(-1) ** k / float(np.prod(np.arange(1, 2 * k + 1, dtype=np.float64))) for k in range(10)]


def sincos(theta):
    """Platform-independent (sin, cos) built from correctly rounded +, -, *.

    Libm / NumPy SIMD sin and cos may differ by an ulp between hosts (x86-64
    and aarch64), which would change the generated polygons.  Quadrant
    reduction by pi/2 (two-part constant) and Taylor polynomials on
    [-pi/4, pi/4] evaluated with separate NumPy multiplies and adds give the
    same bits everywhere (truncation error below 1e-16).
    """
    t = np.asarray(theta, dtype=np.float64)
    q = np.floor(t * (2.0 / np.pi) + 0.5)
    r = (t - q * _HALF_PI_HI) - q * _HALF_PI_LO
    r2 = r * r
    s = np.full_like(r, _SIN_C[-1])
    for c in reversed(_SIN_C[:-1]):
        s = s * r2 + c
    s = s * r
    c_ = np.full_like(r, _COS_C[-1])
    for c in reversed(_COS_C[:-1]):
        c_ = c_ * r2 + c
    k = q.astype(np.int64) & 3
    sin_t = np.select([k == 0, k == 1, k == 2], [s, c_, -s], -c_)
    cos_t = np.select([k == 0, k == 1, k == 2], [c_, -s, -c_], s)
    return sin_t, cos_t


def _angles(rng: np.random.Generator, n: int) -> np.ndarray:
    """n sorted, pairwise distinct U[0, 2pi) draws."""
    th = np.sort(rng.uniform(0.0, TWO_PI, n))
    while True:
        dup = np.flatnonzero(np.diff(th) <= 0.0)
        if dup.size == 0:
            return th
        th[dup + 1] = rng.uniform(0.0, TWO_PI, dup.size)
        th.sort()


def star(n: int, seed: int, centre=(0.0, 0.0), R: float = 1.0) -> np.ndarray:
    """Plain star: radius R*(0.5+0.5u). Returns (n, 2) float64, CCW."""
    rng = np.random.default_rng(seed)
    th = _angles(rng, n)
    r = R * (0.5 + 0.5 * rng.uniform(0.0, 1.0, n))
    sn, cs = sincos(th)
    xy = np.empty((n, 2), dtype=np.float64)
    xy[:, 0] = centre[0] + r * cs
    xy[:, 1] = centre[1] + r * sn
    return xy


def value_noise(theta: np.ndarray, rng: np.random.Generator, base_freq: int,
                octaves: int = 8) -> np.ndarray:
    """Sum of `octaves` periodic 1-D value-noise octaves over theta in [0, 2pi).

    Octave o has base_freq*2^o lattice cells, lattice values U[-1, 1], smoothstep
    interpolation, amplitude 0.5^o.
    """
    g = np.zeros_like(theta)
    amp = 1.0
    for o in range(octaves):
        cells = base_freq << o
        lattice = rng.uniform(-1.0, 1.0, cells)
        t = theta / TWO_PI * cells
        k = np.floor(t).astype(np.int64) % cells
        f = t - np.floor(t)
        s = f * f * (3.0 - 2.0 * f)
        g += amp * (lattice[k] * (1.0 - s) + lattice[(k + 1) % cells] * s)
        amp *= 0.5
    return g


def jagged_star(n: int, seed: int, centre=(0.0, 0.0), R: float = 1.0,
                rotation: float = 0.0, base_freq: int = JAGGED_BASE_FREQ) -> np.ndarray:
    """Jagged star: radius R*(1+0.3g), clamped >= 0.2R, rotated then translated."""
    rng = np.random.default_rng(seed)
    th = _angles(rng, n)
    g = value_noise(th, rng, base_freq)
    r = np.maximum(R * (1.0 + 0.3 * g), 0.2 * R)
    sn, cs = sincos(th + rotation)
    xy = np.empty((n, 2), dtype=np.float64)
    xy[:, 0] = centre[0] + r * cs
    xy[:, 1] = centre[1] + r * sn
    return xy


def pair_small(seed_base: int = 1000):
    """10,000-vertex base at (0,0) and 8,000-vertex overlay at (0.3,0.2)."""
    return star(10_000, seed_base + 0), star(8_000, seed_base + 1, centre=(0.3, 0.2))


# Scale of the large jagged pair.  The reference tests signed areas against an
# absolute EPSILON of 1e-9 (p_seg_tree/util/constants.h:13); at R = 1 the
# million-vertex rings have tangential edges ~6e-6 long whose cross products
# (~4e-11) fall below it, so nearly parallel edges are classified as collinear
# overlaps and the reference's chain handling loops.  R = 1000 keeps every
# area far above the threshold without changing the shape.
LARGE_R = 1000.0


def pair_large(n: int = 1_000_000, seed_base: int = 2000, base_freq: int = JAGGED_BASE_FREQ,
               R: float = LARGE_R):
    """Two n-vertex jagged stars; overlay offset (0.25R, 0.1R) and rotated 0.3 rad."""
    b = jagged_star(n, seed_base + 0, R=R, base_freq=base_freq)
    c = jagged_star(n, seed_base + 1, centre=(0.25 * R, 0.1 * R), R=R, rotation=0.3,
                    base_freq=base_freq)
    return b, c


def one_to_many(n_base: int = 200_000, n_overlays: int = 10_000, seed: int = 3000,
                R: float = LARGE_R, lo: int = 4, hi: int = 5000, rmin: float = 0.001,
                rmax: float = 0.05, near_boundary: float = 0.0):
    """One jagged base and many plain-star overlays (log-uniform sizes and radii)."""
    base = jagged_star(n_base, seed, R=R)
    rng = np.random.default_rng(seed + 1)
    lo_b, hi_b = base.min(axis=0), base.max(axis=0)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi + 1), n_overlays)).astype(np.int64)
    sizes = np.clip(sizes, lo, hi)
    radii = R * np.exp(rng.uniform(np.log(rmin), np.log(rmax), n_overlays))
    centres = rng.uniform(lo_b, hi_b, (n_overlays, 2))
    on_edge = rng.uniform(0.0, 1.0, n_overlays) < near_boundary
    picks = rng.integers(0, n_base, n_overlays)
    centres[on_edge] = base[picks[on_edge]]
    seeds = rng.integers(0, 2**62, n_overlays)
    overlays = [star(int(n), int(s), centre=(float(c[0]), float(c[1])), R=float(r))
                for n, s, c, r in zip(sizes, seeds, centres, radii)]
    return base, overlays


def uneven_pairs(n_pairs: int = 1_000_000, n_large: int = 16, seed: int = 5000, lo: int = 3,
                 hi: int = 2048, large: int = 200_000, chunk: int = 65536):
    """Packed (bxy, boff, cxy, coff) of n_pairs + n_large pairs; the large pairs
    sit at evenly spaced positions."""
    rng = np.random.default_rng(seed)
    total = n_pairs + n_large
    large_at = set(int(round((i + 0.5) * total / max(n_large, 1))) for i in range(n_large))
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi + 1), (total, 2))).astype(np.int64)
    sizes = np.clip(sizes, lo, hi)
    for q in large_at:
        sizes[q] = (large, large)
    boff = np.zeros(total + 1, np.int64)
    coff = np.zeros(total + 1, np.int64)
    boff[1:] = np.cumsum(sizes[:, 0])
    coff[1:] = np.cumsum(sizes[:, 1])
    bxy = np.empty((int(boff[-1]), 2))
    cxy = np.empty((int(coff[-1]), 2))
    centres = rng.uniform(-0.5, 0.5, (total, 2))

    def fill(out, off, p0, p1, centre):
        n = sizes[p0:p1, 0 if out is bxy else 1]
        m = int(n.sum())
        seg = np.repeat(np.arange(p1 - p0), n)
        k = np.arange(m) - np.repeat(off[p0:p1] - off[p0], n)
        th = TWO_PI * (k + rng.uniform(0.0, 1.0, m)) / np.repeat(n, n)
        r = 0.5 + 0.5 * rng.uniform(0.0, 1.0, m)
        sl = slice(int(off[p0]), int(off[p1]))
        out[sl, 0] = centre[seg, 0] + r * np.cos(th)
        out[sl, 1] = centre[seg, 1] + r * np.sin(th)

    zero = np.zeros((total, 2))
    for p0 in range(0, total, chunk):
        p1 = min(total, p0 + chunk)
        fill(bxy, boff, p0, p1, zero[p0:p1])
        fill(cxy, coff, p0, p1, centres[p0:p1])
    for i, q in enumerate(sorted(large_at)):
        b, c = pair_large(large, seed_base=seed + 10 * i)
        bxy[boff[q]:boff[q + 1]] = b
        cxy[coff[q]:coff[q + 1]] = c
    return bxy, boff, cxy, coff


def small_pairs(npairs: int, seed: int = 4000, lo: int = 4, hi: int = 64):
    """Independent small pairs: sizes U[lo, hi], r=0.5+0.5u, overlay centre U[-0.5,0.5]^2."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(npairs):
        nb, nc = rng.integers(lo, hi + 1, 2)
        off = rng.uniform(-0.5, 0.5, 2)
        s = int(rng.integers(0, 2**62))
        out.append((star(int(nb), s), star(int(nc), s + 1, centre=(off[0], off[1]))))
    return out


def ring(n: int, rng: np.random.Generator, centre, r_lo: float, r_hi: float,
         clockwise: bool = False) -> np.ndarray:
    """n vertices at stratified angles 2pi (k + u_k) / n, radius U[r_lo, r_hi]:
    adjacent angles at most 4pi / n apart, so for n >= 16 every edge stays
    farther than 0.94 r_lo from the centre."""
    th = TWO_PI * (np.arange(n) + rng.uniform(0.05, 0.95, n)) / n
    r = rng.uniform(r_lo, r_hi, n)
    sn, cs = sincos(th)
    xy = np.empty((n, 2), dtype=np.float64)
    xy[:, 0] = centre[0] + r * cs
    xy[:, 1] = centre[1] + r * sn
    return xy[::-1].copy() if clockwise else xy


def holed(n: int, seed: int, centre=(0.0, 0.0), R: float = 1.0, holes: int = 1,
          islands: int = 0, n_hole: int | None = None):
    """Components of one polygon: an outer ring of n vertices, `holes` holes
    (at most 5) and `islands` islands inside the first holes.  Returns a list
    of (m, 2) arrays, the outer ring first."""
    if not 0 <= holes <= 5 or not 0 <= islands <= holes:
        raise ValueError("0 <= islands <= holes <= 5")
    rng = np.random.default_rng(seed)
    n = max(int(n), 16)
    m = max(int(n_hole if n_hole else n // 4), 16)
    comps = [ring(n, rng, centre, 0.7 * R, R)]
    phase = rng.uniform(0.0, TWO_PI)
    for h in range(holes):
        a = phase + TWO_PI * h / max(holes, 1)
        hc = centre if holes == 1 else (centre[0] + 0.35 * R * np.cos(a),
                                        centre[1] + 0.35 * R * np.sin(a))
        comps.append(ring(m, rng, hc, 0.12 * R, 0.2 * R, clockwise=True))
        if h < islands:
            comps.append(ring(m, rng, hc, 0.04 * R, 0.08 * R))
    return comps


def write_poly(path, xy: np.ndarray, sep: str = ",") -> None:
    """Reference text format: count line, then `x<sep>y` per vertex at %.17g."""
    xy = np.asarray(xy, dtype=np.float64)
    with open(path, "w") as f:
        f.write(f"{xy.shape[0]}\n")
        f.write("\n".join(f"{x:.17g}{sep}{y:.17g}" for x, y in xy))
        f.write("\n")


def read_poly(path) -> np.ndarray:
    """Parse the reference text format (`x,y` or `x y` per line)."""
    with open(path) as f:
        n = int(f.readline())
        data = f.read().replace(",", " ").split()
    arr = np.array(data[: 2 * n], dtype=np.float64).reshape(n, 2)
    return arr
