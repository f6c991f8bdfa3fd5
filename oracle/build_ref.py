#!/usr/bin/env python3
"""Build the reference's own CPU (OpenMP) clipping binary into oracle/_ref/.

TEST INFRASTRUCTURE ONLY: the binary built here is the checker and the CPU
baseline, never the product.

Recipe (nothing is written outside oracle/_ref/):

1. Stage the reference's CPU-path sources (``src/clip.cpp``,
   ``p_seg_tree/oacc_segment_tree.cpp``, ``p_seg_tree/util.cpp`` and the headers
   they include) into ``oracle/_ref/src/`` as a scratch copy.  The staged copy is
   git-ignored; it travels to the GPU host so the baseline can be rebuilt there
   (the reference tree itself does not exist on that host).
2. Apply the harness patches to the scratch copy (the reference as shipped
   crashes on every benchmark input):

   * ``realToInt`` (``p_seg_tree/oacc_segment_tree.cpp:203-206``) computes
     ``(int)pow(10,10)`` which overflows; it is made 64-bit:
     ``(LONG)(pow(10, positions) * val)``.
   * ``savePolygon`` (``foster/polyclip.h:861-865``) honours
     ``SBC_REF_PRECISION`` (17 gives bit-exact dumps; default stays 6).
   * the Foster back end's ``UNION`` switch (``foster/polyclip.h:39``), which
     the driver leaves off, is set when ``SBC_REF_UNION`` is in the
     environment (union fixtures for the library's union mode).
   * ``multicore_clipping`` (``src/clip.cpp:1415-2115``) dumps its intermediate
     arrays (raw / unique candidates, intersection records, merged vertex
     arrays, initial labels) when ``SBC_REF_DUMP`` names a file prefix.
3. Link a zero-filling ``malloc`` (``ref_zero_malloc.c``): the reference reads
   uninitialised heap memory (``oacc_segment_tree.cpp:4562-4576``,
   ``segment_tree.h:150-156``); zero-filling makes those reads defined and the
   run deterministic.
4. ``g++ -O2 -fopenmp -ffp-contract=off`` with the CCCL Thrust host headers of
   the CUDA toolkit.
5. Foster's sequential Greiner-Hormann code, the reference's own baseline
   (``lib/optimizedFostersAlgorithm/polyclip.cpp`` with its headers), staged
   unpatched and compiled as shipped (``g++ -O2 -std=c++11``) into
   ``oracle/_ref/foster``: ``foster [-union] P.poly Q.poly R.poly``.  ``-ffp-contract=off`` keeps every FP64 expression
   unfused on hosts whose compilers contract by default (aarch64), matching an
   x86-64 ``-O2`` build.

Usage: ``python oracle/build_ref.py [--ref DIR]`` (default DIR: the
``SBC_REFERENCE_DIR`` environment variable, else ``/root/reference``).
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
STAGE = OUT / "src"

FILES = [
    "src/clip.cpp",
    "p_seg_tree/oacc_segment_tree.cpp",
    "p_seg_tree/util.cpp",
    "p_seg_tree/segment_tree/segment_tree.h",
    "p_seg_tree/segment_tree/node.h",
    "p_seg_tree/segment_tree/edge.h",
    "p_seg_tree/segment_tree/data_types.h",
    "p_seg_tree/util/util.h",
    "p_seg_tree/util/constants.h",
    "p_seg_tree/util/thrust_func.h",
    "foster/polyclip.h",
    "foster/polygon.h",
    "foster/point2D.h",
]

FOSTER_FILES = [
    "lib/optimizedFostersAlgorithm/polyclip.cpp",
    "lib/optimizedFostersAlgorithm/point2D.h",
    "lib/optimizedFostersAlgorithm/polygon.h",
    "lib/optimizedFostersAlgorithm/readSCPolygon.h",
]

DUMP_HELPERS = r'''
// ---- oracle harness: intermediate dumps (enabled by SBC_REF_DUMP=<prefix>) ----
#include <cstdio>
#include <cstdlib>
static FILE *sbc_dump_open(int k, const char *name) {
  const char *p = getenv("SBC_REF_DUMP");
  if (!p) return NULL;
  char buf[4096];
  snprintf(buf, sizeof buf, "%s.%d.%s.txt", p, k, name);
  return fopen(buf, "w");
}
static void sbc_dump_ints(int k, const char *name, const int *a, long n) {
  FILE *f = sbc_dump_open(k, name);
  if (!f) return;
  for (long i = 0; i < n; ++i) fprintf(f, "%d\n", a[i]);
  fclose(f);
}
static void sbc_dump_reals(int k, const char *name, const double *a, long n) {
  FILE *f = sbc_dump_open(k, name);
  if (!f) return;
  for (long i = 0; i < n; ++i) fprintf(f, "%.17g\n", a[i]);
  fclose(f);
}
// ---- end oracle harness ----
'''

# (file, anchor, replacement, occurrence-after-marker or None)
PATCHES = [
    ("p_seg_tree/oacc_segment_tree.cpp",
     "return (int)pow(10, positions) * val;",
     "return (LONG)(pow(10, positions) * val);", None),
    # the back end's UNION switch, off in the reference's driver, settable
    # for union fixtures
    ("foster/polyclip.h",
     "bool UNION = false;",
     "bool UNION = (getenv(\"SBC_REF_UNION\") != nullptr);", None),
    ("foster/polyclip.h",
     "  ofstream to(s);\n",
     "  ofstream to(s);\n  if (getenv(\"SBC_REF_PRECISION\")) to.precision(atoi(getenv(\"SBC_REF_PRECISION\")));\n",
     None),
    ("src/clip.cpp",
     '#include "../foster/polyclip.h"\n',
     '#include "../foster/polyclip.h"\n' + DUMP_HELPERS, None),
    ("src/clip.cpp",
     "    int intersectCountDup = bPolLineIdsDup.size();\n",
     "    int intersectCountDup = bPolLineIdsDup.size();\n"
     "    sbc_dump_ints(cType, \"raw_b\", bPolLineIdsDup.data(), intersectCountDup);\n"
     "    sbc_dump_ints(cType, \"raw_c\", cPolLineIdsDup.data(), intersectCountDup);\n"
     "    sbc_dump_ints(cType, \"raw_t\", intersectTypesDup.data(), intersectCountDup);\n",
     "void multicore_clipping"),
    ("src/clip.cpp",
     "                          bPolLineIds, cPolLineIds, intersectTypes, bPolLineIdsSortedIndex, intersectCount);\n",
     "                          bPolLineIds, cPolLineIds, intersectTypes, bPolLineIdsSortedIndex, intersectCount);\n"
     "    sbc_dump_ints(cType, \"uniq_b\", bPolLineIds, intersectCount);\n"
     "    sbc_dump_ints(cType, \"uniq_c\", cPolLineIds, intersectCount);\n"
     "    sbc_dump_ints(cType, \"uniq_t\", intersectTypes, intersectCount);\n",
     "void multicore_clipping"),
    ("src/clip.cpp",
     "                                    intersectAlphaValuesB, intersectAlphaValuesC);\n",
     "                                    intersectAlphaValuesB, intersectAlphaValuesC);\n"
     "    sbc_dump_reals(cType, \"isect_xy\", intersections, 2L * intersectCount);\n"
     "    sbc_dump_ints(cType, \"isect_ab\", intersectAlphaValuesB, intersectCount);\n"
     "    sbc_dump_ints(cType, \"isect_ac\", intersectAlphaValuesC, intersectCount);\n",
     "void multicore_clipping"),
    ("src/clip.cpp",
     "                                    alphaValuesB, alphaValuesC);\n",
     "                                    alphaValuesB, alphaValuesC);\n"
     "    sbc_dump_reals(cType, \"merged_bxy\", intersectedB, 2L * bIntersectedCount);\n"
     "    sbc_dump_reals(cType, \"merged_cxy\", intersectedC, 2L * cIntersectedCount);\n"
     "    sbc_dump_ints(cType, \"merged_balpha\", alphaValuesB, bIntersectedCount);\n"
     "    sbc_dump_ints(cType, \"merged_calpha\", alphaValuesC, cIntersectedCount);\n"
     "    sbc_dump_ints(cType, \"merged_bnb\", neighborsB, bIntersectedCount);\n"
     "    sbc_dump_ints(cType, \"merged_cnb\", neighborsC, cIntersectedCount);\n",
     "void multicore_clipping"),
    ("src/clip.cpp",
     "                                    bIntersectedCount, cIntersectedCount, bInitLabels, cInitLabels);\n",
     "                                    bIntersectedCount, cIntersectedCount, bInitLabels, cInitLabels);\n"
     "    sbc_dump_ints(cType, \"label_b\", bInitLabels, bIntersectedCount);\n"
     "    sbc_dump_ints(cType, \"label_c\", cInitLabels, cIntersectedCount);\n",
     "void multicore_clipping"),
]


def stage(ref: Path) -> None:
    if STAGE.exists():
        shutil.rmtree(STAGE)
    for rel in FILES + FOSTER_FILES:
        dst = STAGE / rel
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(ref / rel, dst)
    for rel, anchor, repl, after in PATCHES:
        p = STAGE / rel
        text = p.read_text()
        start = 0
        if after is not None:
            start = text.index(after)
        pos = text.find(anchor, start)
        if pos < 0:
            raise SystemExit(f"patch anchor not found in {rel}: {anchor!r}")
        text = text[:pos] + repl + text[pos + len(anchor):]
        p.write_text(text)


def compile_ref() -> Path:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = OUT / "seg"
    cmd = [
        "g++", "-O2", "-fopenmp", "-w", "-ffp-contract=off", "-std=c++17",
        "-DCPU", "-DSAVE", "-DTIME", "-D__device__=",
        "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_OMP",
        f"-I{cuda}/include/cccl", f"-I{cuda}/include",
        f"-I{STAGE}/p_seg_tree/segment_tree",
        str(STAGE / "src/clip.cpp"),
        str(STAGE / "p_seg_tree/oacc_segment_tree.cpp"),
        str(STAGE / "p_seg_tree/util.cpp"),
        str(HERE / "ref_zero_malloc.c"),
        "-o", str(exe),
    ]
    subprocess.run(cmd, check=True)
    return exe


def compile_foster() -> Path | None:
    src = STAGE / "lib/optimizedFostersAlgorithm/polyclip.cpp"
    if not src.exists():
        return None
    exe = OUT / "foster"
    subprocess.run(["g++", "-O2", "-w", "-std=c++11", str(src), "-o", str(exe)], check=True)
    return exe


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--ref", default=os.environ.get("SBC_REFERENCE_DIR", "/root/reference"))
    args = ap.parse_args(argv)
    ref = Path(args.ref)
    OUT.mkdir(parents=True, exist_ok=True)
    if (ref / "src/clip.cpp").exists():
        stage(ref)
    elif not (STAGE / "src/clip.cpp").exists():
        print("reference sources unavailable: nothing to build", file=sys.stderr)
        return 2
    exe = compile_ref()
    print(exe)
    fexe = compile_foster()
    if fexe:
        print(fexe)
    return 0


if __name__ == "__main__":
    sys.exit(main())
