"""The tcgen05 Gram path: bit-exact against the popcount path and the golden results.

Counts are integers; the tensor-core path accumulates 0/1 products in f32,
which is exact while a group holds at most 2^24 rows. The tolerance is zero.
"""

from __future__ import annotations

import json
from importlib import import_module
from pathlib import Path

import numpy as np
import pytest

from tests.conftest import case_input
from tests.helpers import digest_pairs, table_of

pytestmark = pytest.mark.gpu

CASES = [c["name"] for c in json.loads((Path(__file__).parent / "golden" / "cases.json").read_text())["cases"]]


def _k2(pkg, bv_np, method, elem=2):
    import torch

    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine(method=method, tc_elem=elem, small_group=1)
    n_f, n_words = bv_np.shape
    dev = torch.from_numpy(np.ascontiguousarray(bv_np).view(np.int64)).cuda()
    fbv, ldp = eng.gather(dev.data_ptr(), n_words, np.arange(n_f), n_words)
    gen = engm.Level(torch.arange(n_f, dtype=torch.int32, device="cuda")[:, None].contiguous(),
                     torch.ones(n_f, dtype=torch.int32, device="cuda"))
    new, _ = eng.count_level(gen, fbv, ldp, n_words, 1, False, False, n_words * 64)
    assert eng.used_tensor == (method == "tensor")
    return new.rows.cpu().numpy(), new.counts.cpu().numpy()


# 4: A operand staged in tensor memory; 8: the CTA-pair (cta_group::2) kernel; 16: the 256 x 256 kernel
@pytest.mark.parametrize("elem", [2, 1, 2 | 4, 1 | 4, 1 | 8, 2 | 8, 1 | 16, 2 | 16])
@pytest.mark.parametrize("n_f,n_words", [(2, 1), (127, 31), (128, 32), (129, 33), (255, 4), (256, 5), (257, 3),
                                         (300, 65), (513, 6)])
def test_pair_counts_match_popcount(pkg, n_f, n_words, elem):
    rng = np.random.default_rng(n_f * 1000 + n_words)
    bv = rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64).view(np.uint64)
    bv &= rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64).view(np.uint64)  # density 1/4
    want_rows, want = _k2(pkg, bv, "popcount")
    got_rows, got = _k2(pkg, bv, "tensor", elem)
    assert np.array_equal(got_rows, want_rows)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("elem", [2, 1, 1 | 8, 1 | 16, 2 | 16])
def test_counts_exact_up_to_2_24_rows(pkg, elem):
    """All-ones columns over 2^24 - 64 rows: every pair count equals the row count exactly."""
    n_rows = (1 << 24) - 64
    n_words = n_rows // 64
    n_f = 130
    bv = np.full((n_f, n_words), np.uint64(0xFFFFFFFFFFFFFFFF), dtype=np.uint64)
    bv[5, 7] = np.uint64(0)  # one column 64 short: its pairs count n_rows - 64
    rows, counts = _k2(pkg, bv, "tensor", elem)
    want = np.full(len(rows), n_rows, dtype=np.int64)
    want[(rows[:, 0] == 5) | (rows[:, 1] == 5)] = n_rows - 64
    assert len(rows) == n_f * (n_f - 1) // 2
    assert np.array_equal(counts, want)


@pytest.mark.parametrize("elem", [2, 1, 1 | 8, 1 | 16, 2 | 16])
@pytest.mark.parametrize("name", ["implication_plain", "implication_infer", "implication_prune", "plain_small_plain",
                                  "dense_k2_small", "deep_sparse_small", "word_tail_2049", "word_tail_65"])
def test_tensor_engine_matches_golden(pkg, golden_cases, name, elem):
    case = golden_cases[name]
    indptr, items, n_rows = case_input(pkg, case)
    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine(method="tensor", tc_elem=elem, small_group=4)
    got = pkg.apriori(table_of(indptr, items, n_rows), min_support=case["min_support"], max_length=case["max_length"],
                      use_gpu=True, prune_equal_support=case["prune_equal_support"],
                      use_generator_pruning=case["use_generator_pruning"], engine=eng, warn_complexity=False)
    assert digest_pairs(pkg.result_pairs(got, n_rows)) == case["digest"]


def test_dense_bernoulli_tensor_matches_popcount(pkg):
    """A dense workload (several 128-member tiles per group) mined both ways."""
    import torch

    syn = pkg.synthetic
    engm = import_module(pkg.__name__ + ".engine")
    p = np.minimum(syn.dense_k2_probs(400, seed=9) * 3, 0.9)
    bv = syn.bernoulli_bitvecs(syn.bernoulli_thresholds(p), 20_000, seed=5)
    dev = torch.from_numpy(bv.view(np.int64)).cuda().view(torch.uint64)
    a = engm.Engine(method="popcount").mine(dev, 20_000, 0.01, 3).host_levels()
    b = engm.Engine(method="tensor").mine(dev, 20_000, 0.01, 3).host_levels()
    assert len(a) == len(b)
    for (ra, ca), (rb, cb) in zip(a, b):
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb)
