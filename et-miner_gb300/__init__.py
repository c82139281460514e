"""GB300-native exact Apriori counting engine: ET-Miner's ``apriori(..., use_gpu=True, bitvecs=...)`` path.

Public API:
    apriori(...)            drop-in for ET-Miner's ``apriori`` GPU route (bitvecs= or transactions)
    mine(...)               the level driver on device bitvectors (column ids out)
    result_pairs(df, n)     a result as sorted (itemset tuple, count) pairs
    Server                  continuous-batching request loop over resident datasets

The compute path is the C-ABI library ``libetm_gb300.so`` (hand-written
sm_103a CUDA, ``csrc/``); there is no CPU fallback. ``build_library()``
compiles it, ``load_library()`` loads it and raises when it is missing.
"""

from __future__ import annotations

from . import synthetic
from ._lib import build_library, lib_path, load_library

__all__ = ["synthetic", "build_library", "load_library", "lib_path"]


def __getattr__(name):
    # The driver modules import torch; load them on first use.
    if name in ("apriori", "result_pairs", "ProfilingSession"):
        from . import apriori as _a

        return getattr(_a, name)
    if name in ("mine", "MineOutput", "Engine"):
        from . import engine as _e

        return getattr(_e, name)
    if name in ("Server",):
        from . import serve as _s

        return getattr(_s, name)
    raise AttributeError(name)
