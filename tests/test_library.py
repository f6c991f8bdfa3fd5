"""CPU checks of the product boundary: the C-ABI library builds for sm_103a,
loads, and exports every function include/sbclip.h declares; the drop-in CLI
is built.  No compute call is made (there is no GPU here)."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "sbclip.h"


@pytest.fixture(scope="module")
def built():
    import build as pkg_build  # segment-tree-based-clipping_gb300/build.py
    return pkg_build.build()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sbc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("sbc_create", "sbc_destroy", "sbc_clip_one_to_many", "sbc_clip_pair",
                 "sbc_clip_pair_device", "sbc_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(str(built))
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_cli_built(built):
    assert (built.parent / "seg").exists()


def test_python_binding_loads(built):
    import sbclip
    L = sbclip.load_library(built)
    assert L.sbc_version().decode().startswith("sbclip-gb300")


def test_kernel_targets_sm103a(built):
    # the fatbin carries sm_103a code only (a compile-time property; read via
    # the build flags rather than by inspecting the binary)
    import build as pkg_build
    assert pkg_build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
