"""GPU checks of polygons with several components (holes, islands) through
the C ABI (sbc_clip_components, sbc_clip_batch_components, the area
forward/backward with components).

Rings are compared with the rings of the reference's Foster program
(golden_components.npz, 6 significant digits, its output format) and bit for
bit with the oracle's multi-component restatement; a batch whose polygons
are single rings gives the plain batch's rings; the gradient is checked
against central finite differences (h = 1e-7) of the shoelace area of the
GPU rings to 1e-8 relative."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_py as O
import sbclip_gen as gen
from conftest import load_component_cases, rings_equal, text6

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clippers():
    import sbclip
    c = {False: sbclip.Clipper(0), True: sbclip.Clipper(0, union=True)}
    yield c
    for x in c.values():
        x.close()


def _oracle(b, c, union=False):
    return O.rings_of(O.clip_components(b, c, union=union)["overlays"][0])


def test_components_match_foster_fixtures_and_oracle(clippers):
    cases = load_component_cases()
    assert len(cases) >= 72
    for kind, union, b, c, want in cases:
        got = clippers[union].clip_components(b, c)
        assert text6(got) == text6(want), (kind, union)
        assert rings_equal(got, _oracle(b, c, union)), (kind, union)


def _holed_pairs(n, seed, lo=16, hi=200):
    rng = np.random.default_rng(seed)
    pairs = []
    for t in range(n):
        n1, n2 = (int(x) for x in rng.integers(lo, hi + 1, 2))
        hb, hc = int(rng.integers(0, 4)), int(rng.integers(0, 3))
        b = gen.holed(n1, seed * 1000 + 2 * t, R=1.0, holes=hb, islands=int(rng.integers(0, hb + 1)))
        ctr = tuple(rng.uniform(-0.4, 0.4, 2))
        c = gen.holed(n2, seed * 1000 + 2 * t + 1, centre=ctr, R=float(rng.uniform(0.5, 1.0)),
                      holes=hc, islands=int(rng.integers(0, hc + 1)))
        pairs.append((b, c))
    return pairs


@pytest.mark.parametrize("union", [False, True])
def test_component_batch_matches_oracle(clippers, union):
    pairs = _holed_pairs(300, 31 + union)
    rings, st = clippers[union].clip_batch_components([b for b, _ in pairs],
                                                      [c for _, c in pairs])
    assert (st == 0).all()
    for (b, c), got in zip(pairs, rings):
        assert rings_equal(got, _oracle(b, c, union))


def test_large_component_pair_stays_in_the_batch_engine(clippers):
    # polygons far above the small/large split: the batch engine clips them
    b = gen.holed(6000, 77, R=1.0, holes=3, islands=2, n_hole=1500)
    c = gen.holed(5000, 78, centre=(0.2, -0.15), R=0.95, holes=2, islands=1, n_hole=1200)
    got = clippers[False].clip_components(b, c)
    assert rings_equal(got, _oracle(b, c))
    assert clippers[False].batch_info()["large_pairs"] == 0


def test_single_ring_components_equal_plain_batch(clippers):
    pairs = gen.small_pairs(400, seed=4700)
    cl = clippers[False]
    plain, st0 = cl.clip_batch([b for b, _ in pairs], [c for _, c in pairs])
    comp, st1 = cl.clip_batch_components([[b] for b, _ in pairs], [[c] for _, c in pairs])
    assert (st0 == st1).all()
    for a, b in zip(plain, comp):
        assert rings_equal(a, b)


def test_mixed_batch_of_rings_and_components(clippers):
    cl = clippers[False]
    holed = _holed_pairs(40, 35)
    small = gen.small_pairs(40, seed=4800)
    bases = [x for pr in zip([b for b, _ in holed], [[b] for b, _ in small]) for x in pr]
    ovs = [x for pr in zip([c for _, c in holed], [[c] for _, c in small]) for x in pr]
    rings, st = cl.clip_batch_components(bases, ovs)
    assert (st == 0).all()
    for b, c, got in zip(bases, ovs, rings):
        assert rings_equal(got, _oracle(b, c))


def test_component_offsets_are_checked(clippers):
    import sbclip
    cl = clippers[False]
    b = gen.holed(40, 3, holes=1)
    bad = [b[0], b[1][:2]]
    with pytest.raises(sbclip.SbcError):
        cl.clip_components(bad, [gen.star(12, 4)])


def _shoelace(rings):
    a = 0.0
    for r in rings:
        x, y = r[:, 0], r[:, 1]
        a += 0.5 * float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))
    return a


def test_component_area_and_gradient(clippers):
    torch = pytest.importorskip("torch")
    import sbclip
    cl = clippers[False]
    pairs = _holed_pairs(3, 41, lo=16, hi=24)
    bases, ovs = [b for b, _ in pairs], [c for _, c in pairs]
    bxy, boff, bk = sbclip.pack_components(bases)
    cxy, coff, ck = sbclip.pack_components(ovs)
    dev = "cuda:0"
    t = {k: torch.from_numpy(v).to(dev) for k, v in
         (("bxy", bxy), ("boff", boff), ("cxy", cxy), ("coff", coff), ("bk", bk), ("ck", ck))}
    n = len(pairs)
    area = torch.zeros(n, dtype=torch.float64, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    args = (n, t["bxy"].data_ptr(), t["boff"].data_ptr(), t["cxy"].data_ptr(),
            t["coff"].data_ptr(), t["bk"].data_ptr(), len(bk) - 1, t["ck"].data_ptr(),
            len(ck) - 1)
    cl.area_forward_components_device(*args, area.data_ptr(), st.data_ptr())
    torch.cuda.synchronize()
    assert (st.cpu().numpy() == 0).all()
    rings, _ = cl.clip_batch_components(bases, ovs)
    for p in range(n):
        want = _shoelace(_oracle(bases[p], ovs[p]))
        assert abs(area[p].item() - want) <= 1e-12 * max(1.0, abs(want))
        assert abs(_shoelace(rings[p]) - want) <= 1e-12 * max(1.0, abs(want))
    ga = torch.ones(n, dtype=torch.float64, device=dev)
    gb = torch.zeros_like(t["bxy"])
    gc = torch.zeros_like(t["cxy"])
    cl.area_backward_components_device(*args, ga.data_ptr(), gb.data_ptr(), gc.data_ptr())
    torch.cuda.synchronize()
    gb, gc = gb.cpu().numpy(), gc.cpu().numpy()
    h = 1e-7
    for p in range(n):
        fb, fc = [], []
        for which, P in ((0, bases[p]), (1, ovs[p])):
            for ci, comp in enumerate(P):
                for i in range(len(comp)):
                    for k in range(2):
                        vals = []
                        for sgn in (1.0, -1.0):
                            q = [x.copy() for x in P]
                            q[ci][i, k] += sgn * h
                            bb, cc = (q, ovs[p]) if which == 0 else (bases[p], q)
                            vals.append(_shoelace(cl.clip_components(bb, cc)))
                        (fb if which == 0 else fc).append((vals[0] - vals[1]) / (2 * h))
        an = np.concatenate([gb[boff[p]:boff[p + 1]].ravel(), gc[coff[p]:coff[p + 1]].ravel()])
        fd = np.array(fb + fc)
        scale = max(np.abs(an).max(), abs(area[p].item()))
        assert np.abs(an - fd).max() <= 1e-8 * scale


def test_cli_reads_and_writes_foster_poly_files(tmp_path):
    """`seg P.poly Q.poly R.poly` on multi-component .poly files gives the
    Foster program's result file, text for text."""
    import subprocess
    from pathlib import Path
    exe = Path(__file__).resolve().parents[1] / "segment-tree-based-clipping_gb300" / "_build" / "seg"
    cases = [c for c in load_component_cases() if c[0] == "generic"][:6]
    for i, (kind, union, b, c, want) in enumerate(cases):
        O.write_poly_components(tmp_path / f"p{i}.poly", b)
        O.write_poly_components(tmp_path / f"q{i}.poly", c)
        args = [str(exe), str(tmp_path / f"p{i}.poly"), str(tmp_path / f"q{i}.poly"),
                str(tmp_path / f"r{i}.poly")] + (["--union"] if union else [])
        p = subprocess.run(args, capture_output=True, text=True, timeout=120)
        assert p.returncode == 0, p.stderr
        got = O.parse_rings((tmp_path / f"r{i}.poly").read_text())
        assert text6(got) == text6(want), (kind, union)
