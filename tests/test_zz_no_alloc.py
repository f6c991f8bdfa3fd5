"""GPU check of the allocation-free entry point, sbc_trace_rings_noalloc.

The entry point traces rings from one pair's merged vertex/intersection
lists with its node pools in a file-scope device array, for callers that may
not allocate device memory.  Every case here first runs the ordinary entry
point (sbc_clip_pair, which grows context buffers), takes the merged lists it
exports, and hands device copies of them to the allocation-free entry point
twice in a row; both calls must return exactly the rings sbc_clip_pair
returned (bit for bit, the tolerance of every ring test in this suite), and
every call after the process's first must leave the device's free memory
unchanged (cudaMemGetInfo before and after the call).

The module is named so that pytest collects it last: it must pass both on
its own in a fresh process (the first call does the per-device set-up) and
after every other test has used the device.
"""
from __future__ import annotations

import numpy as np
import pytest

import sbclip_gen as gen
from conftest import load_small_cases, rings_equal

pytestmark = pytest.mark.gpu


def _device(a, torch, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to("cuda:0")


def _merged_lists(clipper, torch):
    """Device copies of the merged lists of the last clipping call."""
    arr = {n: clipper.debug_array(n) for n in ("merged_bxy", "merged_balpha", "label_b",
                                                "merged_cxy", "merged_cnb", "label_c", "uniq_b")}
    dev = {n: _device(arr[n], torch, np.float64 if n.endswith("xy") else np.int32)
           for n in arr if n != "uniq_b"}
    return dev, len(arr["merged_balpha"]), len(arr["merged_cnb"]), len(arr["uniq_b"])


_FIRST_CALL_DONE = [False]


def _call(torch, sbclip, b_d, nb, c_d, nc, dev, n_b, n_c, k, offsets, xy, xy_cap):
    offsets.fill_(-7)
    xy.fill_(float("nan"))
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(0)[0]
    nr, nv = sbclip.trace_rings_noalloc(
        b_d.data_ptr(), nb, c_d.data_ptr(), nc,
        dev["merged_bxy"].data_ptr(), dev["merged_balpha"].data_ptr(), dev["label_b"].data_ptr(), n_b,
        dev["merged_cxy"].data_ptr(), dev["merged_cnb"].data_ptr(), dev["label_c"].data_ptr(), n_c,
        k, offsets.data_ptr(), offsets.numel(), xy.data_ptr(), xy_cap)
    free_after = torch.cuda.mem_get_info(0)[0]
    # The first call of the process may load the library's device module
    # (and with it the static scratch array) and looks up the array's
    # address; from then on a call must leave the device's free memory as
    # it found it: no allocation, no pool growth.
    if _FIRST_CALL_DONE[0]:
        assert free_after == free_before, (free_before, free_after)
    _FIRST_CALL_DONE[0] = True
    off = offsets[: nr + 1].cpu().numpy()
    pts = xy[: 2 * nv].cpu().numpy().reshape(-1, 2)
    assert off[0] == 0 and off[-1] == nv
    return [pts[off[j]:off[j + 1]] for j in range(nr)]


def _cases():
    cases = [(c.kind, c.base, c.overlays[0]) for c in load_small_cases() if len(c.overlays) == 1]
    cases.append(("star-3000", gen.star(3000, 7), gen.star(2500, 8, centre=(0.2, -0.1))))
    cases.append(("star-swapped", gen.star(2500, 8, centre=(0.2, -0.1)), gen.star(3000, 7)))
    return cases


def test_noalloc_trace_matches_clip_pair_twice():
    torch = pytest.importorskip("torch")
    import sbclip
    clipper = sbclip.Clipper(0)
    try:
        n_checked = 0
        for kind, b, c in _cases():
            want = clipper.clip_pair(b, c)
            dev, n_b, n_c, k = _merged_lists(clipper, torch)
            assert n_b + n_c + 4 * k <= sbclip.NOALLOC_MAX_UNITS, kind
            b_d = _device(b, torch, np.float64)
            c_d = _device(c, torch, np.float64)
            offsets = torch.empty(n_b + 17, dtype=torch.int32, device="cuda:0")
            xy_cap = 2 * (n_b + n_c) + 64
            xy = torch.empty(2 * xy_cap, dtype=torch.float64, device="cuda:0")
            for _ in range(2):
                got = _call(torch, sbclip, b_d, len(b), c_d, len(c), dev, n_b, n_c, k,
                            offsets, xy, xy_cap)
                assert rings_equal(got, want), kind
            n_checked += 1
        assert n_checked > 50
    finally:
        clipper.close()


def test_noalloc_rejects_oversize_and_small_outputs():
    torch = pytest.importorskip("torch")
    import sbclip
    clipper = sbclip.Clipper(0)
    try:
        b, c = gen.star(200, 3), gen.star(150, 4, centre=(0.1, 0.1))
        want = clipper.clip_pair(b, c)
        dev, n_b, n_c, k = _merged_lists(clipper, torch)
        b_d = _device(b, torch, np.float64)
        c_d = _device(c, torch, np.float64)
        offsets = torch.empty(n_b + 17, dtype=torch.int32, device="cuda:0")
        xy = torch.empty(2 * 4 * (n_b + n_c), dtype=torch.float64, device="cuda:0")
        # beyond the stated maximum: rejected on the host before any device work
        with pytest.raises(sbclip.SbcError) as e:
            _call(torch, sbclip, b_d, len(b), c_d, len(c), dev, n_b, n_c,
                  sbclip.NOALLOC_MAX_UNITS // 4, offsets, xy, 4 * (n_b + n_c))
        assert e.value.code == 1 and "limit" in str(e.value)
        # an offsets buffer below n_slots_b + 17 ints is rejected
        short = offsets[: n_b]
        with pytest.raises(sbclip.SbcError) as e:
            _call(torch, sbclip, b_d, len(b), c_d, len(c), dev, n_b, n_c, k, short, xy,
                  4 * (n_b + n_c))
        assert e.value.code == 1
        # too little room for the vertices: the error names the count needed
        nv_need = sum(len(r) for r in want)
        assert nv_need > 1
        with pytest.raises(sbclip.SbcError) as e:
            _call(torch, sbclip, b_d, len(b), c_d, len(c), dev, n_b, n_c, k, offsets, xy,
                  nv_need - 1)
        assert e.value.code == 1 and str(nv_need) in str(e.value)
        # and the next well-formed call is still exact
        got = _call(torch, sbclip, b_d, len(b), c_d, len(c), dev, n_b, n_c, k, offsets, xy,
                    4 * (n_b + n_c))
        assert rings_equal(got, want)
    finally:
        clipper.close()
