"""The per-level flush and resume through apriori() on the GPU (gpu/row_split.py:511-606, 1172-1178).

The files of a flushed mine must hold exactly the itemsets and supports the
in-memory frame holds; a mine resumed from level k must write exactly the
levels above k that the uninterrupted mine wrote. Tolerance: none (supports
are count / N in float64 on both sides, counts come back by rint).
"""

from __future__ import annotations

import shutil
from importlib import import_module
from pathlib import Path

import numpy as np
import pytest

from oracle import miner
from tests.helpers import bitvecs_of, table_of

pytestmark = pytest.mark.gpu

MODES = {"plain": {}, "prune": {"prune_equal_support": True}, "infer": {"use_generator_pruning": True}}


@pytest.fixture(scope="module")
def flush(pkg):
    return import_module(pkg.__name__ + ".flush")


@pytest.fixture(scope="module")
def data(pkg):
    return pkg.synthetic.plain_small(n_rows=20_000, n_items=300, seed=5)


def _levels(flush, d: Path) -> dict[int, list]:
    out = {}
    for p in sorted(Path(d).glob("frequent_k*.parquet")):
        k = int(p.stem.split("frequent_k")[1])
        items, sup = flush.read_level(p)
        out[k] = sorted(zip(map(tuple, items.tolist()), sup.tolist()))
    return out


def _pairs_by_k(pairs, n_rows):
    out = {}
    for s, c in pairs:
        out.setdefault(len(s), []).append((tuple(s), c / n_rows))
    return {k: sorted(v) for k, v in out.items()}


@pytest.mark.parametrize("mode", list(MODES))
def test_flushed_files_hold_the_frame(pkg, flush, data, tmp_path, mode):
    t = data
    kw = dict(min_support=0.005, use_gpu=True, warn_complexity=False, **MODES[mode])
    frame = pkg.apriori(table_of(t.indptr, t.items, t.n_rows), **kw)
    empty = pkg.apriori(table_of(t.indptr, t.items, t.n_rows), output_dir=str(tmp_path), **kw)
    assert len(pkg.result_pairs(empty, t.n_rows)) == 0
    files = _levels(flush, tmp_path)
    want = _pairs_by_k(pkg.result_pairs(frame, t.n_rows), t.n_rows)
    assert len(want) >= 3 and files == want


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("resume_from_k", [2, 3])
def test_resumed_mine_writes_the_uninterrupted_levels(pkg, flush, data, tmp_path, mode, resume_from_k):
    t = data
    kw = dict(min_support=0.005, use_gpu=True, warn_complexity=False, **MODES[mode])
    full, resumed = tmp_path / "full", tmp_path / "resumed"
    pkg.apriori(table_of(t.indptr, t.items, t.n_rows), output_dir=str(full), **kw)
    resumed.mkdir()
    for k in range(1, resume_from_k + 1):
        shutil.copy(flush.level_path(full, k), flush.level_path(resumed, k))
    pkg.apriori(table_of(t.indptr, t.items, t.n_rows), output_dir=str(resumed), resume_from_k=resume_from_k, **kw)
    a, b = _levels(flush, full), _levels(flush, resumed)
    assert max(a) > resume_from_k + 1, "the workload must leave levels to resume"
    assert a == b
    # The uninterrupted files against the oracle (plain mode: every frequent itemset).
    if mode == "plain":
        ref, items = miner.mine_transactions(t.indptr, t.items, t.n_rows, 0.005)
        got = sorted((s, round(sup * t.n_rows)) for k in a for s, sup in a[k])
        assert got == sorted(miner.canonical(ref.levels, items))


def test_bitvecs_route_resume_with_wide_ids(pkg, flush, data, tmp_path):
    """UInt64 ids beyond Int64 through the flush and back (core/result.py:30-54)."""
    import torch

    t = data
    bv, col_to_item = bitvecs_of(t.indptr, t.items, t.n_rows)
    base = (1 << 63) + 101
    wide = {c: base + 3 * int(v) for c, v in col_to_item.items()}
    dev = torch.from_numpy(bv.view(np.int64)).cuda().view(torch.uint64)
    kw = dict(min_support=0.005, warn_complexity=False, use_generator_pruning=True)
    frame = pkg.apriori(bitvecs=(dev, wide, t.n_rows), **kw)
    full, resumed = tmp_path / "full", tmp_path / "resumed"
    pkg.apriori(bitvecs=(dev, wide, t.n_rows), output_dir=str(full), **kw)
    resumed.mkdir()
    shutil.copy(flush.level_path(full, 2), flush.level_path(resumed, 2))
    pkg.apriori(bitvecs=(dev, wide, t.n_rows), output_dir=str(resumed), resume_from_k=2, **kw)
    a, b = _levels(flush, full), _levels(flush, resumed)
    assert a == _pairs_by_k(pkg.result_pairs(frame, t.n_rows), t.n_rows)
    assert {k: v for k, v in a.items() if k > 2} == {k: v for k, v in b.items() if k > 2}
    assert all(s[0] >= base for s, _ in a[3])


def test_resume_at_or_past_the_last_level_writes_nothing(pkg, flush, data, tmp_path):
    t = data
    kw = dict(min_support=0.005, use_gpu=True, warn_complexity=False, max_length=3)
    pkg.apriori(table_of(t.indptr, t.items, t.n_rows), output_dir=str(tmp_path), **kw)
    before = {p.name: p.stat().st_mtime_ns for p in tmp_path.iterdir()}
    assert sorted(before) == [f"frequent_k{k}.parquet" for k in (1, 2, 3)]
    pkg.apriori(table_of(t.indptr, t.items, t.n_rows), output_dir=str(tmp_path), resume_from_k=3, **kw)
    assert {p.name: p.stat().st_mtime_ns for p in tmp_path.iterdir()} == before
    with pytest.raises(FileNotFoundError):
        pkg.apriori(table_of(t.indptr, t.items, t.n_rows), output_dir=str(tmp_path / "none"), resume_from_k=2, **kw)
