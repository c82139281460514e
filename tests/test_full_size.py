"""Full-size workloads checked through size-independent properties (GB300).

The wide-vocabulary workload (1M transactions x 50,000 Zipf items, log-normal
rows, min_support 0.004, int64 ids and again with UInt64 ids near 2^63) and the
deep sparse workload (20M transactions x 2,000 items from planted patterns,
min_support 0.005, max_length 16, generator pruning) are mined at their full
sizes; the oracle cannot run them, so the result is checked by properties that
hold at any size, against counts recomputed independently in PyTorch (AND of
the columns' words and a SWAR popcount):

- every count of a sample of emitted itemsets (stratified by level) is exact;
- emitted itemsets are frequent, ascending and unique;
- closure: every (k-1)-subset of a sampled emitted itemset is emitted with a
  count at least as large (frequent itemsets and generators are both closed
  under subsets);
- completeness on a sample: an extension of an emitted itemset by a larger
  frequent item that is frequent (and, under generator pruning, free: smaller
  than each of its (k-1)-subsets' counts) is emitted;
- level 1 is complete: every column whose popcount reaches min_count is emitted.

Generating the deep sparse workload takes minutes on the host, so these run
when ETM_FULL_SIZE=1 is set (`ETM_FULL_SIZE=1 python -m pytest tests/test_full_size.py -m gpu`).
"""

from __future__ import annotations

import math
import os
from fractions import Fraction
from importlib import import_module

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow,
              pytest.mark.skipif(os.environ.get("ETM_FULL_SIZE") != "1", reason="set ETM_FULL_SIZE=1")]

SAMPLE = 300


def _popcount64(x):
    x = x - ((x >> 1) & 0x5555555555555555)
    x = (x & 0x3333333333333333) + ((x >> 2) & 0x3333333333333333)
    x = (x + (x >> 4)) & 0x0F0F0F0F0F0F0F0F
    return (x * 0x0101010101010101) >> 56


class Recount:
    """Counts of column sets over device bitvectors, computed with plain PyTorch ops."""

    def __init__(self, bv):
        self.bv = bv  # torch int64 [n_cols, W]

    def __call__(self, cols) -> int:
        acc = self.bv[int(cols[0])].clone()
        for c in cols[1:]:
            acc &= self.bv[int(c)]
        return int(_popcount64(acc).sum().item())


def _mine(pkg, indptr, items, n_rows, **kw):
    """Mine through apriori() and return {itemset (column tuple): count}, the column of each item id and
    the device bitvectors of the same columns."""
    api = import_module(pkg.__name__ + ".api")
    cols_of, inv = np.unique(items, return_inverse=True)
    n_cols = len(cols_of)
    bv, _ = api.build_device_bitvecs(indptr, inv.astype(np.int32), n_cols, n_rows, keep_rows=True)
    table = _Csr(indptr, items)
    df = pkg.apriori(table, use_gpu=True, warn_complexity=False, **kw)
    sets = df.itemsets() if isinstance(df, api.ItemsetFrame) else [tuple(s) for s in df.to_arrow().column("itemset").to_pylist()]
    sup = np.asarray(df.support if isinstance(df, api.ItemsetFrame) else df.to_arrow().column("support").to_numpy())
    counts = np.rint(sup * n_rows).astype(np.int64)
    col = {int(v): i for i, v in enumerate(cols_of.tolist())}
    out = {}
    for s, c in zip(sets, counts):
        key = tuple(col[int(x)] for x in s)
        assert key not in out, "duplicate itemset"
        assert list(key) == sorted(key), "items not ascending"
        out[key] = int(c)
    return out, col, bv


class _Csr:
    """The CSR input form apriori() accepts (indptr, items)."""

    def __init__(self, indptr, items):
        self.indptr, self.items = indptr, items


def _check(result, bv, n_rows, min_support, generators, seed):
    rng = np.random.default_rng(seed)
    recount = Recount(bv)
    mc = max(1, math.ceil(Fraction(str(min_support)) * n_rows))
    by_k = {}
    for s, c in result.items():
        assert c >= mc
        by_k.setdefault(len(s), []).append(s)
    # Level 1 complete.
    pc = _popcount64(bv).sum(dim=1).cpu().numpy()
    freq1 = {i for i in range(len(pc)) if pc[i] >= mc}
    emitted1 = {s[0] for s in by_k.get(1, [])}
    if generators:
        freq1 = {i for i in freq1 if pc[i] < n_rows}  # an item in every row is not a generator
    assert emitted1 == freq1
    for i in emitted1:
        assert result[(i,)] == pc[i]
    frequent_items = np.array(sorted(emitted1), dtype=np.int64)
    per_level = max(1, SAMPLE // max(1, len(by_k)))
    checked = 0
    for k, sets in sorted(by_k.items()):
        pick = rng.choice(len(sets), size=min(per_level, len(sets)), replace=False)
        for p in pick:
            s = sets[p]
            assert recount(s) == result[s], s
            for d in range(k if k > 1 else 0):
                sub = s[:d] + s[d + 1:]
                assert sub in result and result[sub] >= result[s], (s, sub)
            # Completeness: extend by a larger frequent item.
            larger = frequent_items[frequent_items > s[-1]]
            if len(larger) == 0:
                continue
            y = s + (int(rng.choice(larger)),)
            cy = recount(y)
            if cy < mc:
                continue
            if generators:
                subs = [y[:d] + y[d + 1:] for d in range(len(y))]
                if any(sub not in result for sub in subs):
                    continue  # a subset is not a frequent generator, so y is not one either
                if any(result[sub] == cy for sub in subs):
                    continue  # not free
            assert y in result and result[y] == cy, y
            checked += 1
    return checked


def test_wide_vocab_full_size(pkg):
    import torch

    syn = pkg.synthetic
    t = syn.wide_vocab(n_rows=1_000_000, n_items=50_000, seed=0)
    result, col, bv = _mine(pkg, t.indptr, t.items, t.n_rows, min_support=0.004)
    assert len(result) > 0
    _check(result, bv, t.n_rows, 0.004, False, seed=1)
    # UInt64 ids near 2^63: the same itemsets under the shifted ids, the same counts.
    big = (np.uint64(2**63 - 1) + t.items.astype(np.uint64)).astype(np.uint64)
    result64, col64, _ = _mine(pkg, t.indptr, big, t.n_rows, min_support=0.004)
    assert result64 == result
    del bv
    torch.cuda.empty_cache()


def test_deep_sparse_full_size(pkg):
    syn = pkg.synthetic
    t = syn.deep_sparse(n_rows=20_000_000, seed=0)
    result, col, bv = _mine(pkg, t.indptr, t.items, t.n_rows, min_support=0.005, max_length=16,
                            use_generator_pruning=True)
    assert max(len(s) for s in result) >= 3
    _check(result, bv, t.n_rows, 0.005, True, seed=2)
