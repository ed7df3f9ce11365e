"""The C ABI library loads and exports every entry point declared in the header."""
import ctypes
import sys
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "athena_gb300.h")
LIB = os.path.join(ROOT, "athena-gamma_gb300", "libathena_gb300.so")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(athg_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared()
    assert "athg_stage" in names and "athg_create" in names
    import athg
    assert set(names) == set(athg.EXPORTS)


def test_library_exports_all_symbols():
    if not os.path.exists(LIB):
        sys.path.insert(0, ROOT)
        import __graft_entry__ as ge  # noqa
        ge.build_library()
    L = ctypes.CDLL(LIB)
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing


def test_create_without_gpu_fails_cleanly():
    import athg
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(athg.AthgError):
        athg.Sim((8, 8, 8), (8, 8, 8), mhd=False, solver="hllc")
