"""Regenerate the golden fixtures from the reference's own CPU route.

Runs ONLY where the ET-Miner sources are present: ETM_REFERENCE_SRC names their
``src`` directory (the one holding ``et_miner/``). polars and loguru are not
needed by the counting code and are stubbed at import time; the package
``__init__`` is bypassed so that cupy is never imported. The reference's
``_k1_seed`` + ``_mine_levels`` (core/cpu_miner.py:973-981, 1066-1161) mine
each case from a TransactionCSR built the way ``build_transaction_csr``
(core/cpu_miner.py:275-308) builds it. The fixtures hold the inputs of the
small cases, the generator and seed of the larger ones, and every case's
digest and per-level sizes; small cases also hold every (itemset, count).

Usage:
    ETM_REFERENCE_SRC=<ET-Miner checkout>/src python tests/golden/make_golden.py   # writes tests/golden/cases.json
"""

from __future__ import annotations

import importlib.util
import json
import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))



def _reference_src() -> Path:
    src = os.environ.get("ETM_REFERENCE_SRC")
    if not src:
        raise SystemExit("set ETM_REFERENCE_SRC to the ET-Miner sources' src directory (the one holding et_miner/)")
    return Path(src)


def _load_reference():
    """Import et_miner.core.cpu_miner from the reference sources with polars/loguru stubbed."""
    REF = _reference_src()

    class _Any:
        def __getattr__(self, name):
            return _Any()

        def __call__(self, *a, **k):
            return _Any()

    pl = types.ModuleType("polars")
    pl.__getattr__ = lambda name: _Any()  # type: ignore[attr-defined]
    sys.modules.setdefault("polars", pl)
    lg = types.ModuleType("loguru")
    lg.logger = _Any()  # type: ignore[attr-defined]
    sys.modules.setdefault("loguru", lg)
    for name, sub in (("et_miner", "et_miner"), ("et_miner.core", "et_miner/core")):
        pkg = types.ModuleType(name)
        pkg.__path__ = [str(REF / sub)]  # type: ignore[attr-defined]
        sys.modules[name] = pkg
    spec = importlib.util.spec_from_file_location("et_miner.core.cpu_miner", REF / "et_miner/core/cpu_miner.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["et_miner.core.cpu_miner"] = mod
    spec.loader.exec_module(mod)
    return mod


def _graft_pkg():
    import __graft_entry__ as g

    return g.package()


def run_reference(cm, indptr, items, n_rows, min_support, max_length, prune, infer):
    """Mine with the reference CPU route; returns (levels as (item-id sets, counts), n_candidates per level)."""
    from oracle.miner import transaction_csr

    csr = transaction_csr(indptr, items, n_rows, min_support)
    if csr is None:
        return [], []
    tc = cm.TransactionCSR(csr.indptr.astype(np.int64), csr.cols.astype(np.int32), n_rows, list(csr.items), csr.counts, len(csr.items))
    gen, prev, emitted = cm._k1_seed(tc, prune)
    mc = cm._mining_min_count(min_support, n_rows)
    max_tx = int(np.diff(indptr).max()) if n_rows else 0
    eff = min(max_length if max_length else float("inf"), max_tx, tc.n_cols)
    cands = [tc.n_cols]

    def cb(k, n_cand, n_freq, ms):
        cands.append(int(n_cand))

    if len(gen):
        cm._mine_levels(tc, gen, prev, emitted, mc, eff, prune, infer, True, cb, None, None, 1)
    levels = [(np.asarray(csr.items)[s], np.asarray(c, dtype=np.int64)) for s, c in emitted if len(s)]
    return levels, cands


def _four_rows():
    rows = [[1, 2, 3], [2, 3, 4], [1, 3, 5], [2, 3]]
    return rows


def _boundary_cone():
    return [[0, 1, 2]] * 700 + [[1, 2]] * 9300


def _implication(seed: int = 3, n_rows: int = 3000, n_items: int = 70):
    """Items >= 6 imply item % 6: many non-free itemsets, prefix groups wider than one tile."""
    rng = np.random.default_rng(seed)
    w = 1.0 / np.arange(1, n_items + 1) ** 0.9
    w /= w.sum()
    rows = []
    for _ in range(n_rows):
        its = set(rng.choice(n_items, size=int(rng.integers(2, 9)), replace=False, p=w).tolist())
        its |= {i % 6 for i in list(its) if i >= 6}
        rows.append(sorted(its))
    return rows


def _csr(rows):
    lens = np.array([len(r) for r in rows], dtype=np.int64)
    indptr = np.zeros(len(rows) + 1, dtype=np.int64)
    np.cumsum(lens, out=indptr[1:])
    items = np.array([x for r in rows for x in r], dtype=np.int64)
    return indptr, items, len(rows)


def _word_tail_rows(n_rows: int, seed: int):
    """Dense small rows over 12 items whose row count leaves a partial last word."""
    rng = np.random.default_rng(seed)
    m = rng.random((n_rows, 12)) < np.linspace(0.9, 0.2, 12)
    return [sorted(np.flatnonzero(r).tolist()) for r in m]


def main() -> None:
    cm = _load_reference()
    pkg = _graft_pkg()
    syn = pkg.synthetic
    from oracle.miner import digest

    cases = []

    def add(name, source, indptr, items, n_rows, s, max_length=None, prune=False, infer=False, full=True, store_rows=None):
        levels, cands = run_reference(cm, indptr, items, n_rows, s, max_length, prune, infer)
        entry = {
            "name": name,
            "source": source,
            "n_rows": int(n_rows),
            "min_support": s,
            "max_length": max_length,
            "prune_equal_support": prune,
            "use_generator_pruning": infer,
            "digest": digest(levels),
            "level_sizes": [int(len(x)) for x, _ in levels],
            "n_itemsets": int(sum(len(x) for x, _ in levels)),
        }
        if store_rows is not None:
            entry["rows"] = store_rows
        if full:
            entry["itemsets"] = [[list(map(int, r)), int(c)] for x, cs in levels for r, c in zip(x, cs)]
        cases.append(entry)
        print(f"{name:40s} levels={entry['level_sizes']} n={entry['n_itemsets']}")

    for prune, infer in ((False, False), (True, False), (False, True)):
        tag = "prune" if prune else ("infer" if infer else "plain")
        r = _four_rows()
        add(f"four_rows_{tag}", "rows", *_csr(r), 0.5, prune=prune, infer=infer, store_rows=r)
        r = _four_rows()
        add(f"four_rows_s025_{tag}", "rows", *_csr(r), 0.25, prune=prune, infer=infer, store_rows=r)
        r = _implication()
        add(f"implication_{tag}", "rows", *_csr(r), 0.01, prune=prune, infer=infer, store_rows=r)
    r = _boundary_cone()
    add("boundary_cone", "rows", *_csr(r), 0.07, store_rows=r)
    add("single_row", "rows", *_csr([[3, 5, 9]]), 0.5, store_rows=[[3, 5, 9]])
    add("item_in_every_row_prune", "rows", *_csr([[1, 2], [1, 3], [1, 2, 3], [1]]), 0.25, prune=True,
        store_rows=[[1, 2], [1, 3], [1, 2, 3], [1]])
    add("full_support", "rows", *_csr([[1, 2], [1, 2], [1, 2, 7]]), 1.0, store_rows=[[1, 2], [1, 2], [1, 2, 7]])
    add("none_frequent", "rows", *_csr([[1], [2], [3], [4]]), 0.5, store_rows=[[1], [2], [3], [4]])
    for n in (1, 31, 63, 64, 65, 127, 129, 2049):
        r = _word_tail_rows(n, seed=n)
        add(f"word_tail_{n}", "rows", *_csr(r), 0.3, store_rows=r)
        add(f"word_tail_{n}_maxlen3", "rows", *_csr(r), 0.3, max_length=3, store_rows=r)

    # plain_small (60,000 rows, Zipf 1.1, s = 0.01) in the three modes.
    t = syn.plain_small()
    for prune, infer in ((False, False), (True, False), (False, True)):
        tag = "prune" if prune else ("infer" if infer else "plain")
        add(f"plain_small_{tag}", {"gen": "plain_small", "seed": 0}, t.indptr, t.items, t.n_rows, 0.01,
            prune=prune, infer=infer, full=(tag == "plain"))
    # Small instances of the other workloads.
    p = syn.dense_k2_probs(256, seed=1)
    bv = syn.bernoulli_bitvecs(syn.bernoulli_thresholds(p), 20_000, seed=7)
    t = syn.bitvecs_to_transactions(bv, 20_000)
    add("dense_k2_small", {"gen": "dense_k2", "n_items": 256, "p_seed": 1, "n_rows": 20_000, "hash_seed": 7},
        t.indptr, t.items, t.n_rows, 0.002, max_length=3, full=False)
    t = syn.deep_sparse(n_rows=200_000, seed=0)
    add("deep_sparse_small", {"gen": "deep_sparse", "n_rows": 200_000, "seed": 0}, t.indptr, t.items, t.n_rows,
        0.005, max_length=16, infer=True, full=False)
    add("deep_sparse_small_prune", {"gen": "deep_sparse", "n_rows": 200_000, "seed": 0}, t.indptr, t.items,
        t.n_rows, 0.005, max_length=16, prune=True, full=False)
    t = syn.wide_vocab(n_rows=100_000, seed=0)
    add("wide_vocab_small", {"gen": "wide_vocab", "n_rows": 100_000, "seed": 0}, t.indptr, t.items, t.n_rows,
        0.004, full=False)

    out = HERE / "cases.json"
    out.write_text(json.dumps({"generator": "tests/golden/make_golden.py", "cases": cases}, separators=(",", ":")))
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
