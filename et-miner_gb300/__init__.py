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


_LAZY = {
    "apriori": "api", "result_pairs": "api", "ProfilingSession": "api", "ItemsetFrame": "api",
    "mine": "engine", "MineOutput": "engine", "Engine": "engine",
    "Server": "serve",
}


def __getattr__(name):
    # The engine, API and serving modules import torch; load them on first use.
    mod = _LAZY.get(name)
    if mod is None:
        raise AttributeError(name)
    import importlib

    return getattr(importlib.import_module(f"{__name__}.{mod}"), name)
