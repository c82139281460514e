"""Test helpers shared by the GPU parity tests."""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from oracle import miner


@dataclass
class CSRInput:
    """A transaction list column as a CSR (what apriori() accepts besides polars/pyarrow frames)."""

    indptr: np.ndarray
    items: np.ndarray


def digest_pairs(pairs) -> str:
    """The golden digest of sorted (itemset, count) pairs."""
    per_k: dict[int, list] = {}
    for s, c in pairs:
        per_k.setdefault(len(s), []).append((s, c))
    levels = []
    for k in sorted(per_k):
        sets = np.array([s for s, _ in per_k[k]], dtype=np.int64).reshape(-1, k)
        counts = np.array([c for _, c in per_k[k]], dtype=np.int64)
        levels.append((sets, counts))
    return miner.digest(levels)


def table_of(indptr, items, n_rows) -> CSRInput:
    return CSRInput(np.asarray(indptr, np.int64), np.asarray(items, np.int64))


def bitvecs_of(indptr, items, n_rows):
    """(host uint64 bitvectors over every distinct item, col -> item dict)."""
    uniq, inv = np.unique(items, return_inverse=True)
    cols = inv.astype(np.int32)
    bv = miner.bitvecs_from_csr(indptr, cols, len(uniq), n_rows)
    return bv, {c: int(v) for c, v in enumerate(uniq)}
