"""The C-ABI library: it builds for sm_103a, loads without a GPU, and exports every declared entry point."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

HEADER = Path(__file__).resolve().parent.parent / "include" / "etm.h"


def declared_symbols() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(etm_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ("etm_build_bitvecs", "etm_popcount_cols", "etm_level_groups", "etm_count_tiles",
                 "etm_count_cands", "etm_level_compact", "etm_level_subsets", "etm_classify"):
        assert name in syms


def test_library_builds_and_exports(pkg):
    path = pkg.build_library()
    assert path.exists()
    raw = ctypes.CDLL(str(path))
    missing = [s for s in declared_symbols() if not hasattr(raw, s)]
    assert not missing, f"declared in etm.h but not exported: {missing}"


def test_bound_signatures_cover_header(pkg):
    from importlib import import_module

    lib_mod = import_module(pkg.__name__ + "._lib")
    assert set(declared_symbols()) <= set(lib_mod.SIGNATURES), set(declared_symbols()) - set(lib_mod.SIGNATURES)


def test_bound_argument_counts_match_header(pkg):
    """Every binding passes as many arguments as its declaration takes (a missing one would shift the rest)."""
    from importlib import import_module

    lib_mod = import_module(pkg.__name__ + "._lib")
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    decls = re.findall(r"\b(?:int|void|const char\s*\*)\s+(etm_[a-z0-9_]+)\s*\(([^;]*?)\)\s*;", text)
    assert len(decls) >= len(declared_symbols()) - 1
    wrong = []
    for name, args in decls:
        args = args.strip()
        n = 0 if args in ("", "void") else args.count(",") + 1
        bound = lib_mod.SIGNATURES[name][1]
        if bound is not None and len(bound) != n:
            wrong.append((name, n, len(bound)))
    assert not wrong, wrong


def test_loads_and_reports_version(pkg):
    lib = pkg.load_library()
    assert lib.etm_version() >= 1
    assert isinstance(lib.etm_last_error(), bytes)


def test_argument_errors_need_no_gpu(pkg):
    """Host-side guards reject bad arguments before any launch (gpu/kernels/loader.py:40-141)."""
    lib = pkg.load_library()
    assert lib.etm_build_bitvecs(None, None, 0, None, 0, 100, 4, 1, None, None) == 1  # ld < ceil(100/64)
    assert b"ld" in lib.etm_last_error()
    assert lib.etm_gather_cols(None, 8, None, 1, 8, None, 30, None) == 1  # out_ld not a multiple of 32
    assert lib.etm_level_groups(None, 10, 0, None, None, None, None, None, 100, None) == 1  # width 0


def test_no_cpu_fallback(pkg, monkeypatch):
    """Without a CUDA device the engine refuses to run instead of computing on the host."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        pkg.mine(None, 10, 0.5)
