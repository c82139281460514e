"""The transactions input on CPU: the device-side frequent-CSR build (run here with torch on the CPU) equals
the host restatement for int64 and UInt64 ids, repeated items and empty rows."""

from __future__ import annotations

from importlib import import_module

import numpy as np
import pytest


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("mc", [1, 3, 50])
def test_device_frequent_csr_matches_host(pkg, wide, mc):
    api = import_module(pkg.__name__ + ".api")
    rng = np.random.default_rng(mc + 10 * wide)
    n_rows = 500
    lens = rng.integers(0, 12, n_rows)
    lens[::37] = 0
    indptr = np.zeros(n_rows + 1, np.int64)
    np.cumsum(lens, out=indptr[1:])
    ids = rng.integers(0, 60, int(lens.sum()))  # repeats inside a row are dropped
    if wide:
        flat = (np.uint64(2**63 - 30) + ids.astype(np.uint64)).astype(np.uint64)  # straddles 2^63
    else:
        flat = (ids * 1_000_003 - 7_000_000).astype(np.int64)  # negative ids too
    rp_h, cols_h, items_h = api._frequent_csr(indptr, flat, n_rows, mc)
    rp_d, cols_d, items_d, row_len, support = api._frequent_csr_device(indptr, flat, n_rows, mc, "cpu")
    assert items_d.dtype == items_h.dtype
    assert np.array_equal(items_d, items_h)
    assert np.array_equal(rp_d.numpy(), rp_h)
    assert np.array_equal(cols_d.numpy(), cols_h)
    assert np.array_equal(row_len, np.diff(rp_h))
    assert np.array_equal(support, np.bincount(cols_h, minlength=len(items_h)))


def test_sort_free_coding_declines_before_any_kernel(pkg):
    """The sort-free coding hands UInt64 ids, non-integer values, empty inputs and id spans past 2^26 to the
    sorting path; all of these are decided before the library is called (here, on the CPU)."""
    api = import_module(pkg.__name__ + ".api")
    rp = np.array([0, 2, 3], np.int64)
    assert api._coded_csr_device(rp, np.array([1, 2, 3], np.uint64), 2, 1, "cpu") is None
    assert api._coded_csr_device(rp, np.array([1.0, 2.0, 3.0]), 2, 1, "cpu") is None
    assert api._coded_csr_device(np.zeros(3, np.int64), np.zeros(0, np.int64), 2, 1, "cpu") is None
    assert api._coded_csr_device(rp, np.array([-5, 2, (1 << 26) - 5], np.int64), 2, 1, "cpu") is None
    assert api.CODE_SPAN_MAX == 1 << 26


@pytest.mark.parametrize("kw,exc,match", [
    (dict(min_support=1.5), ValueError, r"\[0.0, 1.0\]"),
    (dict(min_support="0.1"), TypeError, "numeric"),
    (dict(min_support=True), TypeError, "numeric"),
    (dict(min_support=0.1, max_length=0), ValueError, ">= 1"),
    (dict(min_support=0.1, max_length=2.0), TypeError, "int or None"),
    (dict(min_support=0.1, batch_size=0), ValueError, ">= 1"),
    (dict(min_support=0.1, sparse=True), ValueError, "sparse= was removed"),
    (dict(min_support=0.1, gpu_resident=True), ValueError, "gpu_resident"),
    (dict(min_support=0.1, sparse_from_k=3), ValueError, "sparse_from_k"),
    (dict(min_support=0.1, prune_apriori=False), ValueError, "prune_apriori"),
    (dict(min_support=0.1, streaming=True), ValueError, "streaming"),
    (dict(min_support=0.1, output_dir="gs://bucket/run"), ValueError, "local directory"),
    (dict(min_support=0.1, resume_from_k=2), ValueError, "needs output_dir"),
    (dict(min_support=0.1, anchor_items={1}), ValueError, "anchor_items"),
])
def test_parameter_checks_need_no_gpu(pkg, kw, exc, match):
    """The reference's parameter checks (core/apriori.py:64-106) and the rejected routes raise before any
    device work, with the reference's exception types."""
    with pytest.raises(exc, match=match):
        pkg.apriori([[1, 2], [2, 3]], use_gpu=True, **kw)


def test_non_integer_items_are_coded_by_rank(pkg):
    """Strings, floats and categorical values are coded to ranks among the distinct items (the reference's
    _coded_items, core/apriori.py:277-284), nulls dropped; mixed kinds are refused."""
    api = import_module(pkg.__name__ + ".api")
    rows = [["milk", "bread"], None, ["eggs", None, "bread"], ["milk"]]
    indptr, codes, _, labels = api._list_column(rows, "items")
    assert list(labels) == ["bread", "eggs", "milk"]
    assert indptr.tolist() == [0, 2, 2, 4, 5]
    assert [labels[c] for c in codes] == ["milk", "bread", "eggs", "bread", "milk"]
    indptr, codes, _, labels = api._list_column({"items": [[2.5, 1.0], [1.0]]}, "items")
    assert labels.dtype == np.float64 and list(labels) == [1.0, 2.5] and codes.tolist() == [1, 0, 0]
    indptr, ids, _, labels = api._list_column([[3, 1], [2]], "items")
    assert labels is None and ids.tolist() == [3, 1, 2]
    with pytest.raises(TypeError, match="must all be integers"):
        api._list_column([[1, "a"]], "items")


def test_categorical_pyarrow_items_come_back_as_strings(pkg):
    pa = pytest.importorskip("pyarrow")
    api = import_module(pkg.__name__ + ".api")
    dict_type = pa.dictionary(pa.int32(), pa.string())
    values = pa.array(["b", "a", "b", "c"]).cast(dict_type)
    col = pa.LargeListArray.from_arrays(pa.array([0, 2, 4], pa.int64()), values)
    indptr, codes, _, labels = api._list_column(pa.table({"items": col}), "items")
    assert list(labels) == ["a", "b", "c"] and codes.tolist() == [1, 0, 1, 2]
