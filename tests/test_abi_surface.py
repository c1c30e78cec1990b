"""CPU-side checks of the drop-in boundary: liblcr.so loads and exports every
entry point include/lcr.h declares (no compute call is made)."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols() -> list[str]:
    text = (ROOT / "include" / "lcr.h").read_text()
    return sorted(set(re.findall(r"LCR_API\s+[^;(]*?\b(lcr_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("lcr_icp", "lcr_voxel_grid", "lcr_sor", "lcr_normals", "lcr_backproject", "lcr_accumulate",
                 "lcr_knn", "lcr_transform", "lcr_ctx_create"):
        assert must in syms


def test_library_exports_every_declared_symbol():
    from lowcost3dreconstruction_gb300 import _lib, build
    build.build_lib()
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from lowcost3dreconstruction_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.exported_symbols())
