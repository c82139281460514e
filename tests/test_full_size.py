"""Full-size workloads checked through size-independent properties (GB300).

The deep sparse workload (20M transactions x 2,000 items from planted
patterns, min_support 0.005, max_length 16, generator pruning) is generated on
the device by the hash-defined pattern generator; the wide-vocabulary workload
(1M transactions x 50,000 Zipf items, log-normal rows, min_support 0.004) by
the host generator, then mined through the transactions route with int64 ids
and again with UInt64 ids near 2^63. The oracle cannot mine these sizes, so the
results are checked by ``verify.check_mine``: sampled counts recomputed in
plain PyTorch, level-1 completeness, subset closure, and completeness/absence
of random extensions. A small slice of the pattern generator is checked bit
for bit against its host restatement, and mined against the oracle.
"""

from __future__ import annotations

from importlib import import_module

import numpy as np
import pytest

from tests.helpers import CSRInput, table_of

pytestmark = pytest.mark.gpu


def _mods(pkg):
    return (import_module(pkg.__name__ + ".engine"), import_module(pkg.__name__ + ".verify"),
            import_module(pkg.__name__ + ".api"))


def _assert_clean(rep):
    assert rep["mismatches"] == 0, rep
    assert rep["level1_complete"] and rep["level1_counts_exact"], rep


def test_pattern_generator_matches_host_and_oracle(pkg):
    """The device pattern generator against its host restatement (every bit of 3,000 rows), then the mine of
    that input against the oracle with generator pruning."""
    import torch

    from oracle import miner

    syn = pkg.synthetic
    lib = pkg.load_library()
    spec = syn.pattern_spec(hash_seed=99)
    n_rows = 3_000
    bv = syn.patterns_bitvecs_device(lib, spec, n_rows)
    rows = syn.patterns_rows_host(spec, n_rows)
    lens = np.array([len(r) for r in rows], np.int64)
    indptr = np.zeros(n_rows + 1, np.int64)
    np.cumsum(lens, out=indptr[1:])
    cols = np.array([x for r in rows for x in sorted(r)], np.int32)
    want = miner.bitvecs_from_csr(indptr, cols, spec.n_items, n_rows)
    got = bv.view(torch.int64).cpu().numpy().view(np.uint64)
    assert np.array_equal(got, want)
    engm, _, _ = _mods(pkg)
    out = engm.Engine().mine(bv, n_rows, 0.02, 16, use_generator_pruning=True)
    ref = miner.mine_bitvecs(want, n_rows, 0.02, 16, use_generator_pruning=True)
    assert miner.canonical([(c, n) for c, n in out.host_levels()]) == miner.canonical(ref.levels)
    assert max(sets.shape[1] for sets, _ in ref.levels) >= 3


def test_deep_sparse_full_size(pkg):
    """20M x 2,000 planted patterns (device-generated), min_support 0.005, max_length 16, generator pruning."""
    import torch

    syn = pkg.synthetic
    lib = pkg.load_library()
    engm, verm, _ = _mods(pkg)
    n_rows = 20_000_000
    bv = syn.patterns_bitvecs_device(lib, syn.pattern_spec(), n_rows)
    out = engm.Engine().mine(bv, n_rows, 0.005, 16, use_generator_pruning=True)
    assert len(out.levels) >= 2  # itemsets of 3 or more items
    rep = verm.check_mine(out, bv, n_rows, generators=True, max_length=16, sample=4_000, seed=2)
    _assert_clean(rep)
    assert rep["extensions_frequent"] > 0
    del bv
    torch.cuda.empty_cache()


def test_wide_vocab_full_size(pkg):
    """1M x 50,000 Zipf(1.0) items, log-normal rows, min_support 0.004; through the transactions route with
    int64 ids and UInt64 ids near 2^63 (the same itemsets under the shifted ids, the same counts)."""
    import torch

    syn = pkg.synthetic
    engm, verm, api = _mods(pkg)
    t = syn.wide_vocab(n_rows=1_000_000, n_items=50_000, seed=0)
    cols_of, inv = np.unique(t.items, return_inverse=True)
    bv, rows = api.build_device_bitvecs(t.indptr, inv.astype(np.int32), len(cols_of), t.n_rows, keep_rows=True)
    out = engm.Engine().mine(bv, t.n_rows, 0.004, None, rows=rows)
    rep = verm.check_mine(out, bv, t.n_rows, sample=4_000, seed=1)
    _assert_clean(rep)
    want = sorted((tuple(int(cols_of[c]) for c in s), int(n)) for sets, counts in out.host_levels()
                  for s, n in zip(sets.tolist(), counts.tolist()))
    df = pkg.apriori(table_of(t.indptr, t.items, t.n_rows), min_support=0.004, use_gpu=True, warn_complexity=False)
    assert sorted(pkg.result_pairs(df, t.n_rows)) == want
    big = (np.uint64(2**63 - 1) + t.items.astype(np.uint64)).astype(np.uint64)
    df64 = pkg.apriori(CSRInput(t.indptr, big), min_support=0.004, use_gpu=True, warn_complexity=False)
    shift = [(tuple(int(x) - (2**63 - 1) for x in s), n) for s, n in pkg.result_pairs(df64, t.n_rows)]
    assert sorted(shift) == want
    del bv
    torch.cuda.empty_cache()
