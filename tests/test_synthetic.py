"""The seeded synthetic workloads on CPU: shapes, sizes and distributions as the workloads are quoted, rows
distinct and ascending, determinism in the seed."""

from __future__ import annotations

import numpy as np
import pytest


def _well_formed(t, n_items_max):
    lens = np.diff(t.indptr)
    assert t.indptr[0] == 0 and t.indptr[-1] == len(t.items) and len(t.indptr) == t.n_rows + 1
    assert (lens >= 0).all()
    rid = np.repeat(np.arange(t.n_rows), lens)
    same_row = rid[1:] == rid[:-1]
    assert (np.diff(t.items)[same_row] > 0).all()  # distinct and ascending within a row
    assert t.items.min() >= 0 and t.items.max() < n_items_max
    return lens


def test_plain_small_shape(pkg):
    syn = pkg.synthetic
    t = syn.plain_small(seed=0)
    lens = _well_formed(t, 1000)
    assert t.n_rows == 60_000
    assert abs(lens.mean() - 9.0) < 0.1  # 1 + Poisson(8)
    counts = np.bincount(t.items, minlength=1000)
    top = np.sort(counts)[::-1]
    assert top[0] > 20 * np.median(counts)  # Zipf(1.1) skew
    t2 = syn.plain_small(seed=0)
    assert np.array_equal(t.items, t2.items) and np.array_equal(t.indptr, t2.indptr)


def test_wide_vocab_lengths_small_sample(pkg):
    syn = pkg.synthetic
    t = syn.wide_vocab(n_rows=50_000, seed=3)
    lens = _well_formed(t, 50_000)
    assert lens.min() >= 1 and lens.max() <= 500
    assert 6 <= np.median(lens) <= 10  # log-normal, median 8


def test_deep_sparse_small_sample(pkg):
    syn = pkg.synthetic
    t = syn.deep_sparse(n_rows=20_000, seed=1)
    lens = _well_formed(t, 2_000)
    assert abs(lens.mean() - 11.0) < 0.3  # 1 + Poisson(10)


def test_dense_k2_probabilities_and_bits(pkg):
    syn = pkg.synthetic
    p = syn.dense_k2_probs(4096, seed=0)
    assert abs(p.mean() - 2 / 32) < 0.004  # Beta(2, 30)
    thr = syn.bernoulli_thresholds(p)
    bv = syn.bernoulli_bitvecs(thr[:64], 4096, seed=12345)
    density = np.unpackbits(bv.view(np.uint8), axis=1).mean(axis=1)
    assert np.abs(density - p[:64]).max() < 0.03
    assert np.array_equal(bv, syn.bernoulli_bitvecs(thr[:64], 4096, seed=12345))


@pytest.mark.parametrize("scale", [0.01])
def test_serving_datasets_and_requests(pkg, scale):
    syn = pkg.synthetic
    ds = syn.serving_datasets(seed=0, scale=scale)
    assert len(ds) == 8
    reqs = syn.serving_requests(256, mean_gap_s=0.05, seed=0)
    assert len(reqs) == 256
    gaps = np.diff([r.arrival_s for r in reqs])
    assert abs(gaps.mean() - 0.05) < 0.01
    assert all(0.002 <= r.min_support <= 0.05 and 2 <= r.max_length <= 8 and 0 <= r.dataset < 8 for r in reqs)
