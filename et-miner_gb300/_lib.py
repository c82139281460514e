"""Build and load the C-ABI library ``libetm_gb300.so`` (hand-written sm_103a CUDA).

The library is compiled in-tree with nvcc, one translation unit per
``csrc/*.cu`` file compiled in parallel, then linked. Every entry point
returns an int status (0 = ok); ``check()`` turns a non-zero status into a
``RuntimeError`` carrying ``etm_last_error()``. Loading fails loudly when
the library is missing: the engine has no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libetm_gb300.so"
ARCH = os.environ.get("ETM_CUDA_ARCH", "103a")

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def lib_path() -> Path:
    return PKG_DIR / LIB_NAME


def _nvcc() -> str:
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def build_library(verbose: bool = False, force: bool = False) -> Path:
    """Compile every ``csrc/*.cu`` for sm_103a and link ``libetm_gb300.so``; returns its path."""
    out = lib_path()
    srcs = _sources()
    deps = srcs + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    if not force and out.exists() and all(out.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return out
    BUILD_DIR.mkdir(exist_ok=True)
    flags = [
        f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}",
        "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
        f"-I{INCLUDE}", f"-I{CSRC}", "--expt-relaxed-constexpr",
    ]

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [_nvcc(), *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as pool:
        objs = list(pool.map(compile_one, srcs))
    tmp = out.with_suffix(".so.tmp")
    cmd = [_nvcc(), f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


# (name, restype, argtypes) of every exported entry point; argtypes None = not bound here.
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_U64 = ctypes.c_uint64
_D = ctypes.c_double

SIGNATURES: dict[str, tuple] = {
    "etm_version": (ctypes.c_int, []),
    "etm_last_error": (ctypes.c_char_p, []),
    "etm_device_sm_count": (ctypes.c_int, []),
    "etm_build_bitvecs": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _I64, _I64, _I64, _P, _P]),
    "etm_popcount_cols": (ctypes.c_int, [_P, _I64, _I64, _I64, _P, _P]),
    "etm_gather_cols": (ctypes.c_int, [_P, _I64, _P, _I32, _I64, _P, _I64, _P]),
    "etm_row_order_keys": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _P, _P, _P]),
    "etm_permute_rows": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _P, _P, _P, _P]),
    "etm_tile_occupancy": (ctypes.c_int, [_P, _I64, _I64, _I64, _P, _I64, _P]),
    "etm_item_codes": (ctypes.c_int, [_P, _P, _I64, _I64, _I64, _I64, _P, _P, _P, _P, _P]),
    "etm_code_histogram": (ctypes.c_int, [_P, _I64, _I64, _P, _P]),
    "etm_bitmap_values": (ctypes.c_int, [_P, _I64, _P, _I64, _P, _P]),
    "etm_kept_lengths": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _P, _P]),
    "etm_synth_bernoulli": (ctypes.c_int, [_P, _I32, _I64, _U64, _P, _I64, _P]),
    "etm_synth_patterns": (ctypes.c_int, [_P, _I32, _P, _I32, _P, _P, _I32, _U64, _I32, _I64, _U64, _P, _I64, _P]),
    "etm_level_groups": (ctypes.c_int, [_P, _I64, _I32, _P, _P, _P, _P, _P, _I64, _P]),
    "etm_classify": (ctypes.c_int, [_P, _I32, _I64, _P, _P, _P, _P, _P, _I64, _I64, _I32, _P, _P, _P]),
    "etm_count_tiles": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _P, _P, _P, _I64, _I64, _P, _I32, _P, _P]),
    "etm_count_cands": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _P, _P, _P, _I64, _I64, _P, _P, _P]),
    "etm_triple_counts_rows": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _I64, _P, _P, _I64, _P, _P, _P, _I64, _I64, _P,
                                              _P, _P]),
    "etm_pair_counts_rows": (ctypes.c_int, [_P, _P, _I64, _P, _I64, _I64, _I64, _P, _P]),
    "etm_prefix_counts": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _I64, _P, _P, _I64, _P]),
    "etm_prefix_rows": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _I64, _P, _P, _P]),
    "etm_prefix_segments": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _I64, _P, _P, _P, _I64, _P]),
    "etm_project": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "etm_project_blocked": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _P, _I64, _P, _P, _P, _I64, _P, _P, _P]),
    "etm_rows_transpose": (ctypes.c_int, [_P, _I64, _I64, _I64, _P, _I64, _P]),
    "etm_project_rows": (ctypes.c_int, [_P, _I64, _I64, _P, _I64, _P, _I32, _P, _P, _P, _I64, _P, _P, _P, _I64, _P,
                                        _P]),
    "etm_count_tiles_proj": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _P, _I32, _P, _P]),
    "etm_count_tiles_tc": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _P, _I32, _P, _P, _P]),
    "etm_count_tiles_tc_sel": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _P, _I32, _I32, _P,
                                              _P, _P, _P]),
    "etm_gram_block_members": (ctypes.c_int, [_I32]),
    "etm_tc_mma_rate": (ctypes.c_int, [_I32, _I64, ctypes.POINTER(_D), _P]),
    "etm_popc_rate": (ctypes.c_int, [_I64, ctypes.POINTER(_D), _P]),
    "etm_set_wait_limits": (ctypes.c_int, [_I64, _I64]),
    "etm_device_status": (ctypes.c_int, [_P]),
    "etm_level_compact": (ctypes.c_int, [_P, _P, _I64, _P, _I32, _P, _P, _P, _I64, _I64, _I32, _P, _P, _I64, _P, _P, _I64, _P]),
    "etm_level_compact_static": (ctypes.c_int, [_P, _P, _I64, _P, _I32, _P, _P, _P, _I64, _I64, _I32, _P, _P, _I64, _P, _P]),
    "etm_count_tiles_split": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _P, _P, _P, _I64, _I64, _I64, _P, _I32,
                                             _P, _P]),
    "etm_count_tiles_sel": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _P, _P, _P, _I64, _I64, _P, _I32, _P, _P,
                                           _P]),
    "etm_count_cands_sel": (ctypes.c_int, [_P, _I64, _I64, _P, _I32, _P, _P, _P, _P, _P, _I64, _I64, _P, _I32, _P, _P,
                                           _P, _I64, _P]),
    "etm_count_tiles_proj_sel": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _P, _I32, _P, _P, _P]),
    "etm_classify_sel": (ctypes.c_int, [_P, _I32, _I64, _P, _P, _P, _P, _P, _I64, _I64, _I32, _I32, _P, _I64, _P, _P,
                                        _I64, _P, _I64, _P, _P, _P, _P]),
    "etm_threshold_bits": (ctypes.c_int, [_P, _P, _I64, _I32, _P, _P]),
    "etm_level_compact_bits": (ctypes.c_int, [_P, _P, _I64, _P, _I32, _P, _P, _P, _I64, _I64, _P, _P, _I64, _P, _P, _I64,
                                              _P]),
    "etm_level_subsets": (ctypes.c_int, [_P, _P, _I64, _I32, _P, _P, _I64, _P, _P, _P]),
    "etm_select_rows": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I32, _P, _P, _P, _P, _I64, _P, _P, _I64, _P]),
}


def load_library() -> ctypes.CDLL:
    """Load ``libetm_gb300.so`` (building it first if absent) and bind every entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not path.exists():
            build_library()
        if not path.exists():
            raise RuntimeError(f"{path} is missing: the GB300 engine has no CPU fallback")
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            if args is not None:
                fn.argtypes = args
        _lib = lib
        return lib


def check(status: int, what: str) -> None:
    """Raise RuntimeError with the library's last error message when ``status`` is non-zero."""
    if status != 0:
        msg = load_library().etm_last_error()
        raise RuntimeError(f"{what} failed (status {status}): {msg.decode() if msg else 'unknown error'}")
