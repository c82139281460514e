"""Shared fixtures: the package (imported from et-miner_gb300/), the golden cases, the gpu marker."""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "cases.json"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")
    config.addinivalue_line("markers", "slow: long-running")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def pkg():
    return __graft_entry__.package()


@pytest.fixture(scope="session")
def golden_cases():
    return {c["name"]: c for c in json.loads(GOLDEN.read_text())["cases"]}


def csr_of_rows(rows):
    lens = np.array([len(r) for r in rows], dtype=np.int64)
    indptr = np.zeros(len(rows) + 1, dtype=np.int64)
    np.cumsum(lens, out=indptr[1:])
    items = np.array([x for r in rows for x in r], dtype=np.int64)
    return indptr, items, len(rows)


def case_input(pkg, case):
    """(indptr, items, n_rows) of a golden case: stored rows, or its seeded generator."""
    src = case["source"]
    if src == "rows":
        return csr_of_rows(case["rows"])
    syn = pkg.synthetic
    if src["gen"] == "plain_small":
        t = syn.plain_small(seed=src["seed"])
    elif src["gen"] == "deep_sparse":
        t = syn.deep_sparse(n_rows=src["n_rows"], seed=src["seed"])
    elif src["gen"] == "wide_vocab":
        t = syn.wide_vocab(n_rows=src["n_rows"], seed=src["seed"])
    elif src["gen"] == "dense_k2":
        p = syn.dense_k2_probs(src["n_items"], seed=src["p_seed"])
        bv = syn.bernoulli_bitvecs(syn.bernoulli_thresholds(p), src["n_rows"], seed=src["hash_seed"])
        t = syn.bitvecs_to_transactions(bv, src["n_rows"])
    else:
        raise KeyError(src["gen"])
    return t.indptr, t.items, t.n_rows
