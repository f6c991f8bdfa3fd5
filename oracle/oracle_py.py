"""ctypes access to the C restatement (libsbc_oracle.so) and to the reference
binary built by build_ref.py.  TEST INFRASTRUCTURE ONLY: imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libsbc_oracle.so"
REF_EXE = HERE / "_ref" / "seg"
FOSTER_EXE = HERE / "_ref" / "foster"

ARRAYS = [
    "raw_b", "raw_c", "raw_t", "uniq_b", "uniq_c", "uniq_t",
    "isect_xy", "isect_ab", "isect_ac",
    "merged_bxy", "merged_cxy", "merged_balpha", "merged_calpha", "merged_bnb", "merged_cnb",
    "label_b", "label_c", "ring_offsets", "ring_xy",
]
REAL_ARRAYS = {"isect_xy", "merged_bxy", "merged_cxy", "ring_xy"}
STATS = ["edges", "elem_count", "tree_size", "cover_total", "leaf_end_total"]
TREE_ARRAYS = ["ea", "leaf_off", "leaf_edge", "cov_off", "cov_edge"]


def build_oracle_lib() -> Path:
    """Compile the C restatement (unfused FP64) into oracle/_build/."""
    LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
    src = HERE / "sbc_oracle.c"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", str(src),
                        "-o", str(LIB_PATH), "-lm"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle_lib()
        L = ctypes.CDLL(str(LIB_PATH))
        L.sbco_clip.restype = ctypes.c_void_p
        L.sbco_clip.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_int]
        L.sbco_status.argtypes = [ctypes.c_void_p]
        L.sbco_set_union.argtypes = [ctypes.c_int]
        L.sbco_message.restype = ctypes.c_char_p
        L.sbco_message.argtypes = [ctypes.c_void_p]
        L.sbco_len.restype = ctypes.c_long
        L.sbco_len.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.sbco_data.restype = ctypes.c_void_p
        L.sbco_data.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.sbco_stat.restype = ctypes.c_long
        L.sbco_stat.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.sbco_free.argtypes = [ctypes.c_void_p]
        L.sbco_tree_len.restype = ctypes.c_long
        L.sbco_tree_len.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.sbco_tree_data.restype = ctypes.c_void_p
        L.sbco_tree_data.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.sbco_segment_intersection.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_void_p] * 2
        L.sbco_clip_components.restype = ctypes.c_void_p
        L.sbco_clip_components.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_int]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"oracle status {status}: {msg}")
        self.status = status


def clip(base: np.ndarray, overlays, union: bool = False) -> dict:
    """Run the restatement (union instead of intersection with `union`).
    Returns {'stats': {...}, 'overlays': [ {name: array} ]}."""
    L = lib()
    L.sbco_set_union(1 if union else 0)
    b = np.ascontiguousarray(base, dtype=np.float64).reshape(-1, 2)
    ovs = [np.ascontiguousarray(o, dtype=np.float64).reshape(-1, 2) for o in overlays]
    cxy = np.ascontiguousarray(np.concatenate(ovs, axis=0))
    sizes = np.array([o.shape[0] for o in ovs], dtype=np.int32)
    run = L.sbco_clip(b.ctypes.data, b.shape[0], cxy.ctypes.data, sizes.ctypes.data, len(ovs))
    return _collect(L, run, len(ovs))


def comps_of(comps):
    """(xy, offsets) of a list of (n_i, 2) component arrays."""
    comps = [np.ascontiguousarray(c, dtype=np.float64).reshape(-1, 2) for c in comps]
    off = np.zeros(len(comps) + 1, dtype=np.int32)
    off[1:] = np.cumsum([c.shape[0] for c in comps])
    return np.ascontiguousarray(np.concatenate(comps, axis=0)), off


def clip_components(base_comps, overlay_comps, union: bool = False) -> dict:
    """The restatement on one base and one overlay given as lists of
    components (holes and islands, Foster's .poly format)."""
    L = lib()
    L.sbco_set_union(1 if union else 0)
    b, bo = comps_of(base_comps)
    c, co = comps_of(overlay_comps)
    run = L.sbco_clip_components(b.ctypes.data, b.shape[0], bo.ctypes.data, len(bo) - 1,
                                 c.ctypes.data, c.shape[0], co.ctypes.data, len(co) - 1)
    return _collect(L, run, 1)


def _collect(L, run, k: int) -> dict:
    try:
        st = L.sbco_status(run)
        if st != 0:
            raise OracleError(st, L.sbco_message(run).decode())
        out = {"stats": {n: L.sbco_stat(run, i) for i, n in enumerate(STATS)}, "overlays": [],
               "tree": {}}
        for w, name in enumerate(TREE_ARRAYS):
            n = L.sbco_tree_len(run, w)
            ptr = L.sbco_tree_data(run, w)
            ct = ctypes.c_double if name == "ea" else ctypes.c_int
            a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), (max(n, 1),))[:n]
            out["tree"][name] = a.copy()
        for ov in range(1, k + 1):
            d = {}
            for w, name in enumerate(ARRAYS):
                n = L.sbco_len(run, ov, w)
                ptr = L.sbco_data(run, ov, w)
                if name in REAL_ARRAYS:
                    a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double)), (max(n, 1),))[:n]
                else:
                    a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_int)), (max(n, 1),))[:n]
                d[name] = a.copy()
            out["overlays"].append(d)
        return out
    finally:
        L.sbco_free(run)


def rings_of(d: dict):
    """List of (n,2) arrays from an overlay result dict."""
    off = d["ring_offsets"]
    xy = d["ring_xy"].reshape(-1, 2)
    return [xy[off[i]:off[i + 1]] for i in range(len(off) - 1)]


def segment_intersection(p1, p2, q1, q2):
    L = lib()
    arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (p1, p2, q1, q2)]
    a = ctypes.c_double()
    b = ctypes.c_double()
    t = L.sbco_segment_intersection(*[x.ctypes.data for x in arrs], ctypes.byref(a), ctypes.byref(b))
    return t, a.value, b.value


# ---------------------------------------------------------------------------
# the reference binary
# ---------------------------------------------------------------------------

def ref_available() -> bool:
    return REF_EXE.exists()


def parse_rings(text: str):
    """Parse the reference's result text (`x y,` lines, `;` closes a ring)."""
    rings, cur = [], []
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        end = line.endswith(";")
        body = line.rstrip(",;").strip()
        if body:
            x, y = body.split()
            cur.append((float(x), float(y)))
        if end:
            rings.append(np.array(cur, dtype=np.float64).reshape(-1, 2))
            cur = []
    return rings


def run_reference(base: np.ndarray, overlays, threads: int = 1, precision: int = 17,
                  dump: bool = False, timeout: float = 600.0, union: bool = False) -> dict:
    """Run oracle/_ref/seg on the polygons (written `x,y` at %.17g).

    Returns {'rings': [list per overlay], 'time_line': [...], 'dumps': {...}}.
    """
    import sys
    sys.path.insert(0, str(HERE.parent / "segment-tree-based-clipping_gb300"))
    import sbclip_gen as gen  # noqa: E402

    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "work").mkdir()
        (td / "results").mkdir()
        gen.write_poly(td / "b.txt", base)
        files = []
        for i, o in enumerate(overlays):
            f = td / f"c{i + 1}.txt"
            gen.write_poly(f, o)
            files.append(str(f))
        env = dict(os.environ)
        env["OMP_NUM_THREADS"] = str(threads)
        env["SBC_REF_PRECISION"] = str(precision)
        if union:
            env["SBC_REF_UNION"] = "1"
        if dump:
            env["SBC_REF_DUMP"] = str(td / "dump")
        p = subprocess.run([str(REF_EXE), str(td / "b.txt"), *files], cwd=td / "work", env=env,
                           capture_output=True, text=True, timeout=timeout)
        if p.returncode != 0:
            raise RuntimeError(f"reference exited {p.returncode}: {p.stderr[-400:]}")
        lines = p.stdout.strip().splitlines()
        time_line = [int(x) for x in lines[-1].split() if x.lstrip('-').isdigit()] if lines else []
        rings = []
        for i in range(len(overlays)):
            rp = td / "results" / f"Fig-def-R{i + 1}.txt"
            rings.append(parse_rings(rp.read_text()) if rp.exists() else [])
        dumps = {}
        if dump:
            for i in range(len(overlays)):
                d = {}
                for name in ARRAYS[:-2]:
                    f = td / f"dump.{i + 1}.{name}.txt"
                    if f.exists():
                        dt = np.float64 if name in REAL_ARRAYS else np.int64
                        txt = f.read_text().split()
                        d[name] = np.array(txt, dtype=dt) if txt else np.zeros(0, dt)
                dumps[i + 1] = d
        return {"rings": rings, "time_line": time_line, "dumps": dumps, "stdout": p.stdout}


def _clip_one(args):
    base, overlay, union = args
    try:
        return 0, rings_of(clip(base, [overlay], union=union)["overlays"][0])
    except OracleError as e:
        return e.status, []


def clip_pairs_parallel(pairs, threads: int | None = None, union: bool = False):
    """[(status, rings)] of the restatement on every (base, overlay) pair, on
    `threads` host threads (default: all host cores).  ctypes releases the
    GIL for the C calls, and the restatement keeps no state between calls
    but the union switch, which is the same for every pair here."""
    from concurrent.futures import ThreadPoolExecutor

    lib()
    args = [(np.ascontiguousarray(b, np.float64), np.ascontiguousarray(c, np.float64), union)
            for b, c in pairs]
    n = max(1, min(threads or os.cpu_count() or 1, len(args)))
    if n == 1:
        return [_clip_one(a) for a in args]
    with ThreadPoolExecutor(n) as ex:
        return list(ex.map(_clip_one, args))


# ---------------------------------------------------------------------------
# Foster's sequential code (the reference's own baseline)
# ---------------------------------------------------------------------------

def foster_available() -> bool:
    return FOSTER_EXE.exists()


def write_poly_components(path, comps) -> None:
    """Foster's .poly format: `x y,` per vertex, `;` after each component."""
    with open(path, "w") as f:
        for xy in comps:
            xy = np.asarray(xy, np.float64).reshape(-1, 2)
            lines = [f"{x:.17g} {y:.17g}" for x, y in xy]
            f.write(",\n".join(lines) + ";\n")


def run_foster(base, overlay, timeout: float = 1800.0, union: bool = False) -> dict:
    """Run oracle/_ref/foster on one pair (stdout discarded): the result rings
    (precision 6, the program's output format) and the wall time in ms.  A
    polygon is one (n, 2) array or a list of component arrays."""
    def comps(p):
        return list(p) if isinstance(p, (list, tuple)) else [p]

    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        write_poly_components(td / "p.poly", comps(base))
        write_poly_components(td / "q.poly", comps(overlay))
        args = [str(FOSTER_EXE)] + (["-union"] if union else [])
        t0 = time.perf_counter()
        p = subprocess.run(args + [str(td / "p.poly"), str(td / "q.poly"), str(td / "r.poly")],
                           stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True,
                           timeout=timeout)
        wall = (time.perf_counter() - t0) * 1e3
        if p.returncode != 0:
            raise RuntimeError(f"foster exited {p.returncode}: {p.stderr[-400:]}")
        text = (td / "r.poly").read_text() if (td / "r.poly").exists() else ""
    return {"rings": parse_rings(text), "ms": wall}
