"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares (no compute call is made here)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^\s*(?:const\s+)?(?:int|void|char|double|uint64_t)\s*\**\s*(pcg_\w+)\s*\(", re.M)


def declared_symbols():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names += DECL.findall(open(h, encoding="utf-8").read())
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("pcg_create", "pcg_destroy", "pcg_initialize", "pcg_solve", "pcg_get_field",
                 "pcg_set_agents", "pcg_get_counts", "pcg_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(pcg):
    lib = ctypes.CDLL(pcg.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header(pcg):
    covered = set(pcg.SIGNATURES) | {"pcg_last_error"}
    # the allocation-free entry point is bound where it is used (its own test)
    assert set(declared_symbols()) <= covered | {n for n in declared_symbols() if n.endswith("_noalloc")}


def test_create_without_gpu_fails_cleanly(pcg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pcg.PcgError) as ei:
        pcg.Solver(pcg.FP32)
    assert ei.value.code == 2
