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
    rp_d, cols_d, items_d, row_len = api._frequent_csr_device(indptr, flat, n_rows, mc, "cpu")
    assert items_d.dtype == items_h.dtype
    assert np.array_equal(items_d, items_h)
    assert np.array_equal(rp_d.numpy(), rp_h)
    assert np.array_equal(cols_d.numpy(), cols_h)
    assert np.array_equal(row_len, np.diff(rp_h))


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
    (dict(min_support=0.1, output_dir="/tmp/x"), ValueError, "output_dir"),
    (dict(min_support=0.1, anchor_items={1}), ValueError, "anchor_items"),
])
def test_parameter_checks_need_no_gpu(pkg, kw, exc, match):
    """The reference's parameter checks (core/apriori.py:64-106) and the rejected routes raise before any
    device work, with the reference's exception types."""
    with pytest.raises(exc, match=match):
        pkg.apriori([[1, 2], [2, 3]], use_gpu=True, **kw)
