"""Build libsbclip.so (sm_103a) and the drop-in `seg` CLI in-tree.

    python segment-tree-based-clipping_gb300/build.py [--force]

Every CUDA translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo --fmad=false`` (no FMA
contraction anywhere: the FP64 geometry must round exactly like the
reference's unfused x86-64 build), then linked into ``_build/libsbclip.so``.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libsbclip.so"
CLI = OUT / "seg"
SOURCES = ["sbc_prims.cu", "sbc_front.cu", "sbc_cand.cu", "sbc_mid.cu", "sbc_back.cu", "sbc_batch.cu", "sbc_pairwise.cu", "sbc_api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = Path(cuda) / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "sbclip.h"]
    flags = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-ffp-contract=off", "-I", str(ROOT / "include")]

    def compile_one(src: str) -> Path:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        if not force and _newer(o, [s, *headers]):
            return o
        cmd = [nvcc(), *flags, "-c", str(s), "-o", str(o)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or not _newer(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    cli_src = PKG / "seg_cli.cpp"
    if cli_src.exists() and (force or not _newer(CLI, [cli_src, LIB, ROOT / "include" / "sbclip.h"])):
        cmd = ["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(cli_src), "-o", str(CLI),
               "-L", str(OUT), "-lsbclip", f"-Wl,-rpath,{OUT}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"seg CLI build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    try:
        print(build(force=a.force, verbose=a.verbose))
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
