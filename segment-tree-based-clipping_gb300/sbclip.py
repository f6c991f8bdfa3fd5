"""Python binding of libsbclip.so (the C ABI in include/sbclip.h) via ctypes.

Mirrors the reference's one entry point, ``seg <base> <overlay...>``
(src/clip.cpp:2117-2130 -> multicore_clipping, src/clip.cpp:1415): a base
polygon and k overlays in, for each overlay the list of intersection rings
out, in the reference's output order.  All computation runs in the CUDA
library; if it cannot be loaded every call raises (there is no CPU path).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libsbclip.so"

SBC_FLAG_TIMING = 1
SBC_FLAG_SERIAL_BACKEND = 2
SBC_FLAG_UNION = 4
SBC_FLAG_ENDPOINT_SORT = 8
SBC_FLAG_WIDE_VERTEX_SORT = 16
BATCH_SHAPE_KEYS = ("front", "cand", "back", "backward", "split")

STATS = ["edges", "elementary_points", "tree_size", "cover_entries", "leaf_end_entries",
         "candidates_tested", "raw_hits", "unique", "slots_b", "slots_c", "serial_backend",
         "work_units", "grid_pairs", "vertex_sort", "outside_cmbr"]
PHASES = ["setup", "elementary", "end_lists", "cover_lists", "candidates_merge", "back_end",
          "device_to_host", "total"]
DEBUG_ARRAYS = {
    "uniq_b": (0, np.int32), "uniq_c": (1, np.int32), "uniq_t": (2, np.int32),
    "isect_xy": (3, np.float64), "isect_ab": (4, np.int32), "isect_ac": (5, np.int32),
    "merged_bxy": (6, np.float64), "merged_cxy": (7, np.float64),
    "merged_balpha": (8, np.int32), "merged_calpha": (9, np.int32),
    "merged_bnb": (10, np.int32), "merged_cnb": (11, np.int32),
    "label_b": (12, np.int32), "label_c": (13, np.int32),
    "elementary": (14, np.float64), "leaf_after": (15, np.int32),
    "leaf_before": (16, np.int32), "leaf_range": (17, np.int32),
}


class SbcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sbclip error {code}: {msg}")
        self.code = code


class _Rings(ctypes.Structure):
    _fields_ = [("nrings", ctypes.c_int), ("nverts", ctypes.c_longlong),
                ("offsets", ctypes.c_void_p), ("xy", ctypes.c_void_p)]


class _Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("flags", ctypes.c_int)]


class _MergedLists(ctypes.Structure):
    _fields_ = [("b_xy", ctypes.c_void_p), ("nb", ctypes.c_int),
                ("c_xy", ctypes.c_void_p), ("nc", ctypes.c_int),
                ("merged_bxy", ctypes.c_void_p), ("merged_balpha", ctypes.c_void_p),
                ("label_b", ctypes.c_void_p), ("n_slots_b", ctypes.c_int),
                ("merged_cxy", ctypes.c_void_p), ("merged_cnb", ctypes.c_void_p),
                ("label_c", ctypes.c_void_p), ("n_slots_c", ctypes.c_int),
                ("n_isect", ctypes.c_int)]


NOALLOC_MAX_UNITS = 262144


class _Batch(ctypes.Structure):
    _fields_ = [("npairs", ctypes.c_int), ("b_xy", ctypes.c_void_p), ("b_off", ctypes.c_void_p),
                ("c_xy", ctypes.c_void_p), ("c_off", ctypes.c_void_p)]


class _BatchRings(ctypes.Structure):
    _fields_ = [("npairs", ctypes.c_int), ("nrings", ctypes.c_longlong),
                ("nverts", ctypes.c_longlong), ("pair_ring", ctypes.c_void_p),
                ("ring_off", ctypes.c_void_p), ("xy", ctypes.c_void_p),
                ("status", ctypes.c_void_p)]


BATCH_MAX_VERTICES = 4096


class AreaGraph:
    """A recorded batch area forward + backward (sbc_area_graph_*)."""

    def __init__(self, clipper, handle):
        self._c, self._h = clipper, handle

    def launch(self, stream: int | None = None) -> None:
        self._c._check(self._c._L.sbc_area_graph_launch(self._h, stream))

    def close(self) -> None:
        if self._h:
            self._c._L.sbc_area_graph_destroy(self._h)
            self._h = None


class _Components(ctypes.Structure):
    _fields_ = [("b_comp", ctypes.c_void_p), ("nb_comp", ctypes.c_longlong),
                ("c_comp", ctypes.c_void_p), ("nc_comp", ctypes.c_longlong)]


def pack_components(polys):
    """(xy, polygon offsets, component offsets) of polygons given as lists of
    (n_i, 2) component arrays (a bare array is one component)."""
    comps, off, comp = [], [0], [0]
    for p in polys:
        parts = list(p) if isinstance(p, (list, tuple)) else [p]
        for c in parts:
            c = np.ascontiguousarray(c, np.float64).reshape(-1, 2)
            comps.append(c)
            comp.append(comp[-1] + len(c))
        off.append(comp[-1])
    xy = np.ascontiguousarray(np.concatenate(comps)) if comps else np.zeros((0, 2))
    return xy, np.array(off, np.int64), np.array(comp, np.int64)


class _PairwiseJob(ctypes.Structure):
    _fields_ = [("b_xy", ctypes.c_void_p), ("nb", ctypes.c_int), ("noverlays", ctypes.c_int),
                ("c_xy", ctypes.c_void_p), ("c_off", ctypes.c_void_p)]


def pack_polygons(polys):
    """Concatenate polygons: (xy (n,2) float64, offsets (len+1,) int64)."""
    arrs = [np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 2) for p in polys]
    off = np.zeros(len(arrs) + 1, dtype=np.int64)
    off[1:] = np.cumsum([a.shape[0] for a in arrs])
    xy = np.ascontiguousarray(np.concatenate(arrs, axis=0)) if arrs else np.zeros((0, 2))
    return xy, off


_lib = None


def load_library(path: str | os.PathLike | None = None):
    """Load libsbclip.so (raises OSError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise OSError(f"libsbclip.so not built at {p}; run segment-tree-based-clipping_gb300/build.py")
    L = ctypes.CDLL(str(p))
    vp, i, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
    L.sbc_create.argtypes = [ctypes.POINTER(_Options), ctypes.POINTER(vp)]
    L.sbc_destroy.argtypes = [vp]
    L.sbc_last_error.argtypes = [vp]
    L.sbc_last_error.restype = ctypes.c_char_p
    L.sbc_clip_one_to_many.argtypes = [vp, vp, i, vp, vp, i, ctypes.POINTER(_Rings), vp]
    L.sbc_clip_pair.argtypes = [vp, vp, i, vp, i, ctypes.POINTER(_Rings), vp]
    L.sbc_clip_pair_device.argtypes = [vp, vp, i, vp, i, ctypes.POINTER(_Rings), vp]
    L.sbc_stats.argtypes = [vp, ctypes.POINTER(ll), i]
    L.sbc_phase_times.argtypes = [vp, ctypes.POINTER(ctypes.c_float), i]
    L.sbc_debug_array.argtypes = [vp, i, vp, ll, ctypes.POINTER(ll)]
    L.sbc_classify_pairs.argtypes = [vp, vp, i, vp, vp, vp, vp, vp]
    L.sbc_kernel_launches.restype = ctypes.c_ulonglong
    L.sbc_profile_end.argtypes = [vp, i, vp, vp, vp, i, ctypes.POINTER(i)]
    L.sbc_profile_timeline.argtypes = [vp, i, vp, vp, vp, i, ctypes.POINTER(i)]
    L.sbc_version.restype = ctypes.c_char_p
    for nm in ("sbc_clip_batch", "sbc_clip_batch_device"):
        getattr(L, nm).argtypes = [vp, ctypes.POINTER(_Batch), ctypes.POINTER(_BatchRings), vp]
    for nm in ("sbc_area_forward", "sbc_area_forward_device"):
        getattr(L, nm).argtypes = [vp, ctypes.POINTER(_Batch), vp, vp, vp]
    for nm in ("sbc_area_backward", "sbc_area_backward_device"):
        getattr(L, nm).argtypes = [vp, ctypes.POINTER(_Batch), vp, vp, vp, vp]
    for nm in ("sbc_clip_batch_components", "sbc_clip_batch_components_device"):
        getattr(L, nm).argtypes = [vp, ctypes.POINTER(_Batch), ctypes.POINTER(_Components),
                                   ctypes.POINTER(_BatchRings), vp]
    L.sbc_clip_components.argtypes = [vp, vp, vp, i, vp, vp, i, ctypes.POINTER(_Rings), vp]
    L.sbc_area_forward_components_device.argtypes = [vp, ctypes.POINTER(_Batch),
                                                     ctypes.POINTER(_Components), vp, vp, vp]
    L.sbc_area_backward_components_device.argtypes = [vp, ctypes.POINTER(_Batch),
                                                      ctypes.POINTER(_Components), vp, vp, vp,
                                                      vp]
    for nm in ("sbc_clip_pairwise", "sbc_clip_pairwise_device"):
        getattr(L, nm).argtypes = [vp, ctypes.POINTER(_PairwiseJob), ctypes.POINTER(_BatchRings),
                                   vp]
    L.sbc_pairwise_info.argtypes = [vp, ctypes.POINTER(ll), i]
    L.sbc_pairwise_area_device.argtypes = [vp, ctypes.POINTER(_PairwiseJob), vp, vp, vp]
    L.sbc_pairwise_area_backward_device.argtypes = [vp, ctypes.POINTER(_PairwiseJob), vp, vp, vp,
                                                    vp]
    L.sbc_batch_set_arena_budget.argtypes = [vp, ll]
    L.sbc_area_graph_create.argtypes = [vp, ctypes.POINTER(_Batch), vp, vp, vp, vp, vp, vp,
                                        ctypes.POINTER(vp)]
    L.sbc_area_graph_launch.argtypes = [vp, vp]
    L.sbc_area_graph_destroy.argtypes = [vp]
    L.sbc_batch_info.argtypes = [vp, ctypes.POINTER(ll), i]
    L.sbc_pairwise_set_cell_factor.argtypes = [vp, ctypes.c_double]
    L.sbc_pairwise_set_split.argtypes = [vp, i]
    L.sbc_pairwise_set_workers.argtypes = [vp, i]
    L.sbc_batch_set_shape.argtypes = [vp, vp]
    L.sbc_batch_get_shape.argtypes = [vp, vp]
    L.sbc_batch_autotune.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    L.sbc_pairwise_get_workers.argtypes = [vp]
    L.sbc_pairwise_autotune.argtypes = [vp, ctypes.POINTER(_PairwiseJob), ctypes.POINTER(i),
                                        ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), vp]
    L.sbc_trace_rings_noalloc.argtypes = [ctypes.POINTER(_MergedLists), vp, i, vp, ll,
                                          ctypes.POINTER(i), ctypes.POINTER(ll), vp,
                                          ctypes.c_char_p, i]
    _lib = L
    return L


def kernel_launches() -> int:
    return int(load_library().sbc_kernel_launches())


def profile_begin() -> None:
    """Start bracketing every library launch with CUDA events."""
    load_library().sbc_profile_begin()


def profile_end(with_bytes: bool = False) -> dict:
    """Stop profiling; {kernel name: (total ms, launches)}, or (total ms,
    launches, algorithmic bytes) with with_bytes."""
    L = load_library()
    cap = 256
    names = ctypes.create_string_buffer(cap * 64)
    ms = (ctypes.c_float * cap)()
    cnt = (ctypes.c_int * cap)()
    by = (ctypes.c_double * cap)()
    n = ctypes.c_int()
    L.sbc_profile_end(names, cap * 64, ms, cnt, by, cap, ctypes.byref(n))
    nm = names.raw.split(b"\0")
    if with_bytes:
        return {nm[i].decode(): (float(ms[i]), int(cnt[i]), float(by[i]))
                for i in range(min(n.value, cap))}
    return {nm[i].decode(): (float(ms[i]), int(cnt[i])) for i in range(min(n.value, cap))}


def profile_timeline() -> list[tuple[str, float, float, int]]:
    """The launches of the window the last profile_end closed, in launch
    order: (kernel name, start ms from the first launch's start, duration ms,
    stream number)."""
    L = load_library()
    n = ctypes.c_int()
    L.sbc_profile_timeline(None, 0, None, None, None, 0, ctypes.byref(n))
    cap = n.value
    if cap <= 0:
        return []
    names = ctypes.create_string_buffer(cap * 64)
    t0 = (ctypes.c_float * cap)()
    dur = (ctypes.c_float * cap)()
    sid = (ctypes.c_int * cap)()
    L.sbc_profile_timeline(names, cap * 64, t0, dur, sid, cap, ctypes.byref(n))
    nm = names.raw.split(b"\0")
    return [(nm[i].decode(), float(t0[i]), float(dur[i]), int(sid[i])) for i in range(cap)]


def _rings_from(r: _Rings):
    n = r.nrings
    if n <= 0:
        return []
    off = np.ctypeslib.as_array(ctypes.cast(r.offsets, ctypes.POINTER(ctypes.c_int)), (n + 1,)).copy()
    nv = int(r.nverts)
    xy = np.ctypeslib.as_array(ctypes.cast(r.xy, ctypes.POINTER(ctypes.c_double)), (2 * nv,)).copy()
    xy = xy.reshape(-1, 2)
    return [xy[off[j]:off[j + 1]] for j in range(n)]


class Clipper:
    """One library context (one CUDA stream, grow-only device buffers)."""

    def __init__(self, device: int = 0, timing: bool = False, serial_backend: bool = False,
                 union: bool = False, endpoint_sort: bool = False,
                 wide_vertex_sort: bool = False):
        """union: every clipping call returns base ∪ overlay instead of base ∩ overlay.
        endpoint_sort: the elementary intervals from the sort of all edge
        endpoints rather than of the vertices (a test hook; same results).
        wide_vertex_sort: the vertex sort on 64-bit keys rather than 32-bit
        keys with the equal-key runs fixed up (a test hook; same results)."""
        self._L = load_library()
        opt = _Options(device, (SBC_FLAG_TIMING if timing else 0) |
                       (SBC_FLAG_SERIAL_BACKEND if serial_backend else 0) |
                       (SBC_FLAG_UNION if union else 0) |
                       (SBC_FLAG_ENDPOINT_SORT if endpoint_sort else 0) |
                       (SBC_FLAG_WIDE_VERTEX_SORT if wide_vertex_sort else 0))
        h = ctypes.c_void_p()
        rc = self._L.sbc_create(ctypes.byref(opt), ctypes.byref(h))
        if rc != 0:
            raise SbcError(rc, "sbc_create failed")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.sbc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise SbcError(rc, self._L.sbc_last_error(self._h).decode())

    def clip(self, base, overlays, stream: int | None = None):
        """Rings of base ∩ overlay_i for every overlay (one segment tree)."""
        b = np.ascontiguousarray(base, dtype=np.float64).reshape(-1, 2)
        ovs = [np.ascontiguousarray(o, dtype=np.float64).reshape(-1, 2) for o in overlays]
        cxy = np.ascontiguousarray(np.concatenate(ovs, axis=0))
        sizes = np.array([o.shape[0] for o in ovs], dtype=np.int32)
        outs = (_Rings * len(ovs))()
        self._check(self._L.sbc_clip_one_to_many(self._h, b.ctypes.data, b.shape[0], cxy.ctypes.data,
                                                 sizes.ctypes.data, len(ovs), outs, stream))
        return [_rings_from(outs[i]) for i in range(len(ovs))]

    def clip_pair(self, base, overlay, stream: int | None = None):
        return self.clip(base, [overlay], stream)[0]

    def clip_pair_flat(self, base, overlay, stream: int | None = None, copy: bool = True):
        """sbc_clip_pair with the result as two arrays: ring offsets
        (nrings+1 int32) and vertices (nverts x 2 float64).  With copy=False
        they are views of the context's result memory, valid until the next
        call on this Clipper (what a C caller of sbc_clip_pair receives)."""
        b = np.ascontiguousarray(base, dtype=np.float64).reshape(-1, 2)
        c = np.ascontiguousarray(overlay, dtype=np.float64).reshape(-1, 2)
        r = _Rings()
        self._check(self._L.sbc_clip_pair(self._h, b.ctypes.data, b.shape[0], c.ctypes.data,
                                          c.shape[0], ctypes.byref(r), stream))
        if r.nrings <= 0:
            return np.zeros(1, np.int32), np.zeros((0, 2))
        off = np.ctypeslib.as_array(ctypes.cast(r.offsets, ctypes.POINTER(ctypes.c_int)),
                                    (r.nrings + 1,))
        xy = np.ctypeslib.as_array(ctypes.cast(r.xy, ctypes.POINTER(ctypes.c_double)),
                                   (2 * int(r.nverts),))
        if copy:
            off, xy = off.copy(), xy.copy()
        return off, xy.reshape(-1, 2)

    def clip_pair_device(self, d_base: int, nb: int, d_overlay: int, nc: int,
                         stream: int | None = None):
        """Device pointers in; returns (nrings, nverts, d_offsets, d_xy) device pointers."""
        r = _Rings()
        self._check(self._L.sbc_clip_pair_device(self._h, d_base, nb, d_overlay, nc,
                                                 ctypes.byref(r), stream))
        return r.nrings, int(r.nverts), r.offsets, r.xy

    # ---- batches of independent pairs (host arrays)
    def _batch(self, bases, overlays):
        if len(bases) != len(overlays):
            raise ValueError("one overlay per base")
        bxy, boff = pack_polygons(bases)
        cxy, coff = pack_polygons(overlays)
        keep = (bxy, boff, cxy, coff)
        b = _Batch(len(bases), bxy.ctypes.data, boff.ctypes.data, cxy.ctypes.data, coff.ctypes.data)
        return b, keep

    def clip_batch(self, bases, overlays, stream: int | None = None):
        """Rings of every pair: (list of ring lists, status array)."""
        b, keep = self._batch(bases, overlays)
        r = _BatchRings()
        self._check(self._L.sbc_clip_batch(self._h, ctypes.byref(b), ctypes.byref(r), stream))
        np_ = len(bases)
        pr = np.ctypeslib.as_array(ctypes.cast(r.pair_ring, ctypes.POINTER(ctypes.c_longlong)),
                                   (np_ + 1,)).copy()
        ro = np.ctypeslib.as_array(ctypes.cast(r.ring_off, ctypes.POINTER(ctypes.c_longlong)),
                                   (int(r.nrings) + 1,)).copy()
        xy = (np.ctypeslib.as_array(ctypes.cast(r.xy, ctypes.POINTER(ctypes.c_double)),
                                    (2 * int(r.nverts),)).copy().reshape(-1, 2)
              if r.nverts > 0 else np.zeros((0, 2)))
        st = np.ctypeslib.as_array(ctypes.cast(r.status, ctypes.POINTER(ctypes.c_int)),
                                   (np_,)).copy() if np_ else np.zeros(0, np.int32)
        out = []
        for p in range(np_):
            out.append([xy[ro[q]:ro[q + 1]] for q in range(pr[p], pr[p + 1])])
        return out, st

    def clip_components(self, base, overlay, stream: int | None = None):
        """Rings of one pair of multi-component polygons (lists of component
        arrays) through sbc_clip_components."""
        bxy, _, bk = pack_components([base])
        cxy, _, ck = pack_components([overlay])
        bk32, ck32 = bk.astype(np.int32), ck.astype(np.int32)
        r = _Rings()
        self._check(self._L.sbc_clip_components(self._h, bxy.ctypes.data, bk32.ctypes.data,
                                                len(bk32) - 1, cxy.ctypes.data, ck32.ctypes.data,
                                                len(ck32) - 1, ctypes.byref(r), stream))
        return _rings_from(r)

    def clip_batch_components(self, bases, overlays, stream: int | None = None):
        """Rings of every pair of multi-component polygons (each a list of
        component arrays, or one array): (list of ring lists, status array)."""
        if len(bases) != len(overlays):
            raise ValueError("one overlay per base")
        bxy, boff, bk = pack_components(bases)
        cxy, coff, ck = pack_components(overlays)
        b = _Batch(len(bases), bxy.ctypes.data, boff.ctypes.data, cxy.ctypes.data,
                   coff.ctypes.data)
        k = _Components(bk.ctypes.data, len(bk) - 1, ck.ctypes.data, len(ck) - 1)
        r = _BatchRings()
        self._check(self._L.sbc_clip_batch_components(self._h, ctypes.byref(b), ctypes.byref(k),
                                                      ctypes.byref(r), stream))
        return self._unpack_rings(r, len(bases))

    def area_forward_components_device(self, npairs, d_bxy, d_boff, d_cxy, d_coff, d_bcomp,
                                       nb_comp, d_ccomp, nc_comp, d_area, d_status=None,
                                       stream: int | None = None):
        b = _Batch(npairs, d_bxy, d_boff, d_cxy, d_coff)
        k = _Components(d_bcomp, nb_comp, d_ccomp, nc_comp)
        self._check(self._L.sbc_area_forward_components_device(
            self._h, ctypes.byref(b), ctypes.byref(k), d_area, d_status, stream))

    def area_backward_components_device(self, npairs, d_bxy, d_boff, d_cxy, d_coff, d_bcomp,
                                        nb_comp, d_ccomp, nc_comp, d_grad_area, d_grad_b,
                                        d_grad_c, stream: int | None = None):
        b = _Batch(npairs, d_bxy, d_boff, d_cxy, d_coff)
        k = _Components(d_bcomp, nb_comp, d_ccomp, nc_comp)
        self._check(self._L.sbc_area_backward_components_device(
            self._h, ctypes.byref(b), ctypes.byref(k), d_grad_area, d_grad_b, d_grad_c, stream))

    @staticmethod
    def _unpack_rings(r, np_):
        pr = np.ctypeslib.as_array(ctypes.cast(r.pair_ring, ctypes.POINTER(ctypes.c_longlong)),
                                   (np_ + 1,)).copy()
        ro = np.ctypeslib.as_array(ctypes.cast(r.ring_off, ctypes.POINTER(ctypes.c_longlong)),
                                   (int(r.nrings) + 1,)).copy()
        xy = (np.ctypeslib.as_array(ctypes.cast(r.xy, ctypes.POINTER(ctypes.c_double)),
                                    (2 * int(r.nverts),)).copy().reshape(-1, 2)
              if r.nverts > 0 else np.zeros((0, 2)))
        st = np.ctypeslib.as_array(ctypes.cast(r.status, ctypes.POINTER(ctypes.c_int)),
                                   (np_,)).copy() if np_ else np.zeros(0, np.int32)
        return [[xy[ro[q]:ro[q + 1]] for q in range(pr[p], pr[p + 1])] for p in range(np_)], st

    def clip_pairwise(self, base, overlays, stream: int | None = None):
        """`seg base overlay_i` for every overlay: (list of ring lists, status array)."""
        cxy, coff = pack_polygons(overlays)
        r = self._pairwise(base, cxy, coff, stream)
        return self._unpack_rings(r, len(overlays))

    def _pairwise(self, base, cxy, coff, stream):
        bxy = np.ascontiguousarray(base, dtype=np.float64).reshape(-1, 2)
        cxy = np.ascontiguousarray(cxy, dtype=np.float64)
        coff = np.ascontiguousarray(coff, dtype=np.int64)
        j = _PairwiseJob(bxy.ctypes.data, bxy.shape[0], len(coff) - 1, cxy.ctypes.data,
                         coff.ctypes.data)
        r = _BatchRings()
        self._check(self._L.sbc_clip_pairwise(self._h, ctypes.byref(j), ctypes.byref(r), stream))
        return r

    def clip_pairwise_flat(self, base, cxy, coff, stream: int | None = None, copy: bool = True):
        """sbc_clip_pairwise on packed overlays (pack_polygons): (pair_ring,
        ring_off, xy, status) arrays; with copy=False, views of the context's
        result memory valid until the next call (what a C caller receives)."""
        r = self._pairwise(base, cxy, coff, stream)
        n = len(coff) - 1

        def view(ptr, ct, count):
            if count <= 0:
                return np.zeros(0, np.int64 if ct is ctypes.c_longlong else
                                (np.int32 if ct is ctypes.c_int else np.float64))
            a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), (count,))
            return a.copy() if copy else a

        return (view(r.pair_ring, ctypes.c_longlong, n + 1),
                view(r.ring_off, ctypes.c_longlong, int(r.nrings) + 1),
                view(r.xy, ctypes.c_double, 2 * int(r.nverts)).reshape(-1, 2),
                view(r.status, ctypes.c_int, n))

    def clip_pairwise_device(self, d_bxy, nb, noverlays, d_cxy, d_coff,
                             stream: int | None = None):
        """Device-array form; returns (nrings, nverts) and leaves the rings on the device."""
        j = _PairwiseJob(d_bxy, nb, noverlays, d_cxy, d_coff)
        r = _BatchRings()
        self._check(self._L.sbc_clip_pairwise_device(self._h, ctypes.byref(j), ctypes.byref(r),
                                                     stream))
        return int(r.nrings), int(r.nverts)

    def area_graph(self, npairs, d_bxy, d_boff, d_cxy, d_coff, d_grad_area, d_grad_b, d_grad_c,
                   d_area=None, d_status=None, stream: int | None = None) -> "AreaGraph":
        """Record the batch's area forward + backward as one CUDA graph."""
        b = _Batch(npairs, d_bxy, d_boff, d_cxy, d_coff)
        h = ctypes.c_void_p()
        self._check(self._L.sbc_area_graph_create(self._h, ctypes.byref(b), d_grad_area, d_grad_b,
                                                  d_grad_c, d_area, d_status, stream,
                                                  ctypes.byref(h)))
        return AreaGraph(self, h)

    def set_batch_arena_budget(self, nbytes: int) -> None:
        self._check(self._L.sbc_batch_set_arena_budget(self._h, int(nbytes)))

    def batch_shape(self) -> dict:
        """The batch engine's knobs: block sizes and the small/large split."""
        v = (ctypes.c_int * 5)()
        self._check(self._L.sbc_batch_get_shape(self._h, v))
        return dict(zip(BATCH_SHAPE_KEYS, list(v)))

    def set_batch_shape(self, **kw) -> None:
        cur = self.batch_shape()
        cur.update(kw)
        v = (ctypes.c_int * 5)(*[int(cur[k]) for k in BATCH_SHAPE_KEYS])
        self._check(self._L.sbc_batch_set_shape(self._h, v))

    def autotune_batch_device(self, npairs, d_bxy, d_boff, d_cxy, d_coff, d_grad_area, d_grad_b,
                              d_grad_c, stream: int | None = None) -> dict:
        """Pick the batch engine's block sizes and split by timing forward +
        backward on this batch (the gradient outputs are overwritten)."""
        b = _Batch(npairs, d_bxy, d_boff, d_cxy, d_coff)
        v = (ctypes.c_int * 5)()
        ms = ctypes.c_double()
        self._check(self._L.sbc_batch_autotune(self._h, ctypes.byref(b), d_grad_area, d_grad_b,
                                               d_grad_c, v, ctypes.byref(ms), stream))
        out = dict(zip(BATCH_SHAPE_KEYS, list(v)))
        out["best_ms"] = ms.value
        return out

    def batch_info(self) -> dict:
        """Shape of the last batch call."""
        v = (ctypes.c_longlong * 2)()
        self._L.sbc_batch_info(self._h, v, 2)
        return {"chunks": v[0], "large_pairs": v[1]}

    def pairwise_area_device(self, d_bxy, nb, noverlays, d_cxy, d_coff, d_area, d_status=None,
                             stream: int | None = None) -> None:
        j = _PairwiseJob(d_bxy, nb, noverlays, d_cxy, d_coff)
        self._check(self._L.sbc_pairwise_area_device(self._h, ctypes.byref(j), d_area, d_status,
                                                     stream))

    def pairwise_area_backward_device(self, d_bxy, nb, noverlays, d_cxy, d_coff, d_grad_area,
                                      d_grad_b, d_grad_c, stream: int | None = None) -> None:
        j = _PairwiseJob(d_bxy, nb, noverlays, d_cxy, d_coff)
        self._check(self._L.sbc_pairwise_area_backward_device(self._h, ctypes.byref(j),
                                                              d_grad_area, d_grad_b, d_grad_c,
                                                              stream))

    def pairwise_info(self) -> dict:
        """Diagnostics of the last pairwise call."""
        v = (ctypes.c_longlong * 5)()
        self._L.sbc_pairwise_info(self._h, v, 5)
        return {"fallback_pairs": v[0], "unique": v[1], "tested": v[2], "grid_cells": v[3],
                "big_pairs": v[4]}

    def set_pairwise_cell_factor(self, f: float) -> None:
        self._check(self._L.sbc_pairwise_set_cell_factor(self._h, float(f)))

    def set_pairwise_split(self, records: int) -> None:
        self._check(self._L.sbc_pairwise_set_split(self._h, int(records)))

    def set_pairwise_workers(self, workers: int) -> None:
        self._check(self._L.sbc_pairwise_set_workers(self._h, int(workers)))

    def pairwise_workers(self) -> int:
        return int(self._L.sbc_pairwise_get_workers(self._h))

    def autotune_pairwise_device(self, d_bxy, nb, noverlays, d_cxy, d_coff,
                                 stream: int | None = None) -> dict:
        """Pick the big-pair split and grid cell width by timing the job."""
        j = _PairwiseJob(d_bxy, nb, noverlays, d_cxy, d_coff)
        sp, cf, ms = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        self._check(self._L.sbc_pairwise_autotune(self._h, ctypes.byref(j), ctypes.byref(sp),
                                                  ctypes.byref(cf), ctypes.byref(ms), stream))
        return {"split": sp.value, "cell_factor": cf.value, "best_ms": ms.value}

    def area_forward(self, bases, overlays, stream: int | None = None):
        """Intersection area of every pair: (area, status)."""
        b, keep = self._batch(bases, overlays)
        area = np.zeros(len(bases), np.float64)
        st = np.zeros(len(bases), np.int32)
        self._check(self._L.sbc_area_forward(self._h, ctypes.byref(b), area.ctypes.data,
                                             st.ctypes.data, stream))
        return area, st

    def area_forward_packed(self, bxy, boff, cxy, coff, stream: int | None = None):
        """sbc_area_forward on packed host arrays (pack_polygons): (area, status)."""
        b = _Batch(len(boff) - 1, bxy.ctypes.data, boff.ctypes.data, cxy.ctypes.data,
                   coff.ctypes.data)
        n = len(boff) - 1
        area = np.zeros(n, np.float64)
        st = np.zeros(n, np.int32)
        self._check(self._L.sbc_area_forward(self._h, ctypes.byref(b), area.ctypes.data,
                                             st.ctypes.data, stream))
        return area, st

    def area_backward_packed(self, bxy, boff, cxy, coff, grad_area, stream: int | None = None):
        """sbc_area_backward on packed host arrays: (grad_b, grad_c) packed like bxy, cxy."""
        b = _Batch(len(boff) - 1, bxy.ctypes.data, boff.ctypes.data, cxy.ctypes.data,
                   coff.ctypes.data)
        ga = np.ascontiguousarray(grad_area, dtype=np.float64)
        gb = np.empty_like(bxy)
        gc = np.empty_like(cxy)
        self._check(self._L.sbc_area_backward(self._h, ctypes.byref(b), ga.ctypes.data,
                                              gb.ctypes.data, gc.ctypes.data, stream))
        return gb, gc

    def area_backward(self, bases, overlays, grad_area, stream: int | None = None):
        """d(sum grad_area * area)/d(vertices): (list of (nb,2), list of (nc,2))."""
        b, keep = self._batch(bases, overlays)
        ga = np.ascontiguousarray(grad_area, dtype=np.float64)
        boff, coff = keep[1], keep[3]
        gb = np.zeros((int(boff[-1]), 2))
        gc = np.zeros((int(coff[-1]), 2))
        self._check(self._L.sbc_area_backward(self._h, ctypes.byref(b), ga.ctypes.data,
                                              gb.ctypes.data, gc.ctypes.data, stream))
        return ([gb[boff[p]:boff[p + 1]] for p in range(len(bases))],
                [gc[coff[p]:coff[p + 1]] for p in range(len(overlays))])

    # ---- device-array variants (pointers from e.g. torch tensors)
    def area_forward_device(self, npairs, d_bxy, d_boff, d_cxy, d_coff, d_area, d_status=None,
                            stream: int | None = None):
        b = _Batch(npairs, d_bxy, d_boff, d_cxy, d_coff)
        self._check(self._L.sbc_area_forward_device(self._h, ctypes.byref(b), d_area, d_status,
                                                    stream))

    def area_backward_device(self, npairs, d_bxy, d_boff, d_cxy, d_coff, d_grad_area, d_grad_b,
                             d_grad_c, stream: int | None = None):
        b = _Batch(npairs, d_bxy, d_boff, d_cxy, d_coff)
        self._check(self._L.sbc_area_backward_device(self._h, ctypes.byref(b), d_grad_area,
                                                     d_grad_b, d_grad_c, stream))

    def stats(self) -> dict:
        arr = (ctypes.c_longlong * len(STATS))()
        self._check(self._L.sbc_stats(self._h, arr, len(STATS)))
        return {n: int(arr[i]) for i, n in enumerate(STATS)}

    def phase_times(self) -> dict:
        arr = (ctypes.c_float * len(PHASES))()
        self._check(self._L.sbc_phase_times(self._h, arr, len(PHASES)))
        return {n: float(arr[i]) for i, n in enumerate(PHASES)}

    def debug_array(self, name: str) -> np.ndarray:
        which, dt = DEBUG_ARRAYS[name]
        cnt = ctypes.c_longlong()
        self._check(self._L.sbc_debug_array(self._h, which, None, 0, ctypes.byref(cnt)))
        out = np.empty(max(cnt.value, 1), dtype=dt)
        self._check(self._L.sbc_debug_array(self._h, which, out.ctypes.data, cnt.value,
                                            ctypes.byref(cnt)))
        return out[:cnt.value]

    def classify(self, pairs):
        """Edge-pair classifier on the device; pairs: (n, 8) p1 p2 q1 q2."""
        p = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1, 8)
        n = p.shape[0]
        t = np.empty(n, np.int32)
        a = np.empty(n, np.float64)
        b = np.empty(n, np.float64)
        ai = np.empty(n, np.int32)
        bi = np.empty(n, np.int32)
        self._check(self._L.sbc_classify_pairs(self._h, p.ctypes.data, n, t.ctypes.data, a.ctypes.data,
                                               b.ctypes.data, ai.ctypes.data, bi.ctypes.data))
        return t, a, b, ai, bi


def trace_rings_noalloc(b_xy: int, nb: int, c_xy: int, nc: int, merged_bxy: int,
                        merged_balpha: int, label_b: int, n_slots_b: int, merged_cxy: int,
                        merged_cnb: int, label_c: int, n_slots_c: int, n_isect: int,
                        ring_offsets: int, offsets_cap: int, ring_xy: int, xy_cap_verts: int,
                        stream: int | None = None):
    """Allocation-free ring tracing (sbc_trace_rings_noalloc): every pointer
    is a device address the caller owns; returns (nrings, nverts).  Raises
    SbcError on a non-zero status."""
    L = load_library()
    m = _MergedLists(b_xy, nb, c_xy, nc, merged_bxy, merged_balpha, label_b, n_slots_b,
                     merged_cxy, merged_cnb, label_c, n_slots_c, n_isect)
    nr = ctypes.c_int()
    nv = ctypes.c_longlong()
    err = ctypes.create_string_buffer(256)
    rc = L.sbc_trace_rings_noalloc(ctypes.byref(m), ring_offsets, offsets_cap, ring_xy,
                                   xy_cap_verts, ctypes.byref(nr), ctypes.byref(nv), stream,
                                   err, 256)
    if rc != 0:
        raise SbcError(rc, err.value.decode())
    return nr.value, nv.value


def format_rings(rings, precision: int = 6) -> str:
    """The reference's result text (foster/polygon.h:576-585): `x y,` per
    vertex, `;` after a ring's last vertex, ostream default precision."""
    fmt = f"%.{precision}g"
    out = []
    for r in rings:
        lines = [f"{fmt % x} {fmt % y}" for x, y in r]
        out.append(",\n".join(lines) + ";\n")
    return "".join(out)
