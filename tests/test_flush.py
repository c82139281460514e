"""The per-level parquet flush: frequent_k{k}.parquet with the reference's schema (io/flush.py:63-140),
written and read by pyarrow where installed and by the built-in codec everywhere (CPU only)."""

from __future__ import annotations

from importlib import import_module

import numpy as np
import pytest


@pytest.fixture(scope="module")
def flush(pkg):
    return import_module(pkg.__name__ + ".flush")


def _level(dtype, n=1000, k=3, seed=0):
    rng = np.random.default_rng(seed)
    if dtype == np.uint64:
        items = (np.uint64(2**63 + 5) + rng.integers(0, 1000, size=(n, k)).astype(np.uint64)).astype(np.uint64)
    else:
        items = rng.integers(0, 50 if dtype == np.int32 else 2**40, size=(n, k)).astype(np.int64)
    sup = rng.integers(1, 10**6, size=n) / 10**6
    return items, sup


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint64])
@pytest.mark.parametrize("n,k", [(1000, 3), (1, 1), (0, 2), (37, 16)])
def test_builtin_round_trip(flush, tmp_path, dtype, n, k):
    items, sup = _level(dtype, n, k)
    p = flush.write_level(tmp_path / "frequent_k3.parquet", items, sup, engine="builtin")
    got_items, got_sup = flush.read_level(p, engine="builtin")
    assert np.array_equal(got_sup, sup)
    if n:
        assert got_items.shape == (n, k)
        assert np.array_equal(got_items.astype(items.dtype), items)
        want_dtype = np.uint64 if dtype == np.uint64 else (np.int32 if dtype == np.int32 else np.int64)
        assert got_items.dtype == want_dtype


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint64])
def test_builtin_files_open_in_pyarrow_and_back(flush, tmp_path, dtype):
    pq = pytest.importorskip("pyarrow.parquet")
    items, sup = _level(dtype)
    p = flush.write_level(tmp_path / "a.parquet", items, sup, engine="builtin")
    table = pq.read_table(str(p))
    assert table.column_names == ["itemset", "support"]
    assert [list(r) for r in table.column("itemset").to_pylist()[:5]] == items[:5].tolist()
    assert np.array_equal(table.column("support").to_numpy(), sup)
    for comp in ("none", "gzip"):
        q = flush.write_level(tmp_path / f"b_{comp}.parquet", items, sup, engine="pyarrow", compression=comp)
        got_items, got_sup = flush.read_level(q, engine="builtin")
        assert np.array_equal(got_items.astype(items.dtype), items) and np.array_equal(got_sup, sup)


def test_reference_compression_needs_pyarrow_to_read(flush, tmp_path):
    pytest.importorskip("pyarrow.parquet")
    items, sup = _level(np.int32)
    p = flush.write_level(tmp_path / "z.parquet", items, sup, engine="pyarrow")  # zstd level 2, as the reference
    with pytest.raises(ValueError, match="needs pyarrow"):
        flush.read_level(p, engine="builtin")
    got_items, got_sup = flush.read_level(p, engine="pyarrow")
    assert np.array_equal(got_items, items) and np.array_equal(got_sup, sup)


# ---- apriori(output_dir=, resume_from_k=): option checks and the resume reader (host only) ----------------------

@pytest.fixture(scope="module")
def api(pkg):
    return import_module(pkg.__name__ + ".api")


def test_flush_options_are_checked(api, tmp_path):
    assert api._check_flush_options(None, None) is False
    assert api._check_flush_options(str(tmp_path), None) is False
    assert api._check_flush_options(tmp_path, 1) is False  # resume_from_k=1 mines from the start
    assert api._check_flush_options(str(tmp_path), 3) is True
    with pytest.raises(ValueError, match="needs output_dir"):
        api._check_flush_options(None, 2)
    with pytest.raises(ValueError, match="local directory"):
        api._check_flush_options("gs://bucket/run", None)
    for bad in (0, -1, True, 2.0):
        with pytest.raises(ValueError, match="positive integer"):
            api._check_flush_options(str(tmp_path), bad)


def test_non_integer_items_refuse_the_flush_before_any_work(pkg, tmp_path):
    """Per-level files and resume store integer ids: string items raise before an engine or CSR exists."""
    rows = [["10", "9", "b"], ["10", "b"]]
    for kw in ({"output_dir": str(tmp_path)}, {"output_dir": str(tmp_path), "resume_from_k": 2}):
        with pytest.raises(ValueError, match="not integer ids"):
            pkg.apriori(rows, min_support=0.5, use_gpu=True, **kw)


@pytest.mark.parametrize("wide", [False, True])
def test_resume_reader_maps_ids_to_columns(api, flush, tmp_path, wide):
    base = 2**63 + 11 if wide else 1000
    dt = np.uint64 if wide else np.int64
    item_of_col = np.array([base + 7, base + 2, base + 5, base + 9], dtype=dt)  # unsorted, as col_to_item may be
    sets = np.array([[base + 7, base + 2], [base + 2, base + 9], [base + 5, base + 9]], dtype=dt)
    counts = np.array([3, 1_999_999_999, 17], dtype=np.int64)
    n_rows = 2_000_000_000
    flush.write_level(flush.level_path(tmp_path, 2), sets, counts / n_rows)
    k, cols, got = api._resume_level(str(tmp_path), 2, item_of_col, n_rows)
    assert k == 2 and np.array_equal(got, counts)
    assert np.array_equal(item_of_col[cols], sets)
    with pytest.raises(FileNotFoundError):
        api._resume_level(str(tmp_path), 3, item_of_col, n_rows)
    with pytest.raises(ValueError, match="not in this input"):
        api._resume_level(str(tmp_path), 2, item_of_col[:3], n_rows)


def test_level_writer_writes_every_level_and_raises_its_errors(api, flush, tmp_path):
    w = api._LevelFlush(str(tmp_path), np.array([5, 6, 7], np.int64), 10)
    w(1, np.array([[0], [2]]), np.array([4, 9]))
    w(2, np.array([[0, 2]]), np.array([3]))
    w.close()
    items, sup = flush.read_level(flush.level_path(tmp_path, 2))
    assert items.tolist() == [[5, 7]] and sup.tolist() == [0.3]
    bad = api._LevelFlush(str(tmp_path / "missing" / "dir"), np.array([5], np.int64), 10)
    bad(1, np.array([[0]]), np.array([4]))
    with pytest.raises(OSError):
        bad.close()
