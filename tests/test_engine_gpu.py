"""GPU parity: the engine through apriori() against the reference's golden results and the oracle.

Every itemset and every count must be identical (bit-exact integer work).
"""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import miner
from tests.conftest import case_input, csr_of_rows
from tests.helpers import bitvecs_of, digest_pairs, table_of

pytestmark = pytest.mark.gpu

CASES = [c["name"] for c in json.loads((Path(__file__).parent / "golden" / "cases.json").read_text())["cases"]]


def _rows_engine(e, k3=False):
    """An engine that counts K=2 (and with ``k3`` K=3) row-wise whenever the transactions are given."""
    e.k2_rows_max_r = float("inf")
    if k3:
        e.k3_rows_max_r = float("inf")
    return e


def _lex_engine(e):
    """An engine whose transactions always take the lex row order (and the tile-occupancy skip)."""
    e.row_order, e.lex_min_rows = "lex", 0
    return e


@pytest.fixture(scope="module")
def engines(pkg):
    from importlib import import_module

    eng = import_module(pkg.__name__ + ".engine")
    return {
        "batched": eng.Engine(form="batched"),
        "plain": eng.Engine(form="plain"),
        "tiny": eng.Engine(form="batched", chunk_cands=97, small_group=3),
        "proj": eng.Engine(form="batched", small_group=2, proj_density=1.01, proj_bytes=1 << 14),
        "noproj": eng.Engine(form="batched", project=False),
        "popcount": eng.Engine(method="popcount"),
        "rows": _rows_engine(eng.Engine()),
        "rows3": _rows_engine(eng.Engine(), k3=True),
        "tuned": eng.Engine(autotune=import_module(pkg.__name__ + ".autotune").Autotuner(min_candidates=1)),
        "dense": eng.Engine(fused=False),
        "dense_tiny": eng.Engine(fused=False, chunk_cands=97, small_group=3),
        "rows_dense": _rows_engine(eng.Engine(fused=False), k3=True),
        "proj_cols": eng.Engine(form="batched", small_group=2, proj_density=1.01, proj_bytes=1 << 14, proj_rows=False),
        "popcount_rows": eng.Engine(method="popcount", small_group=2, proj_density=1.01),
        "lex": _lex_engine(eng.Engine()),
        "lex_proj": _lex_engine(eng.Engine(form="batched", small_group=2, proj_density=1.01, proj_bytes=1 << 14)),
    }


@pytest.mark.parametrize("name", CASES)
def test_transactions_match_golden(pkg, golden_cases, engines, name):
    case = golden_cases[name]
    indptr, items, n_rows = case_input(pkg, case)
    got = pkg.apriori(table_of(indptr, items, n_rows), min_support=case["min_support"], max_length=case["max_length"],
                      use_gpu=True, prune_equal_support=case["prune_equal_support"],
                      use_generator_pruning=case["use_generator_pruning"], engine=engines["batched"],
                      warn_complexity=False)
    pairs = pkg.result_pairs(got, n_rows)
    assert digest_pairs(pairs) == case["digest"], name
    if "itemsets" in case:
        want = sorted(((tuple(s), c) for s, c in case["itemsets"]), key=lambda t: (len(t[0]), t[0]))
        assert pairs == want


@pytest.mark.parametrize("form", ["plain", "tiny", "proj", "noproj", "popcount", "tuned", "rows", "rows3", "dense",
                                  "dense_tiny", "rows_dense", "proj_cols", "popcount_rows", "lex", "lex_proj"])
@pytest.mark.parametrize("name", ["implication_plain", "implication_prune", "implication_infer", "plain_small_plain",
                                  "deep_sparse_small", "dense_k2_small", "word_tail_65"])
def test_forms_match_golden(pkg, golden_cases, engines, name, form):
    case = golden_cases[name]
    indptr, items, n_rows = case_input(pkg, case)
    got = pkg.apriori(table_of(indptr, items, n_rows), min_support=case["min_support"], max_length=case["max_length"],
                      use_gpu=True, prune_equal_support=case["prune_equal_support"],
                      use_generator_pruning=case["use_generator_pruning"], engine=engines[form],
                      warn_complexity=False)
    assert digest_pairs(pkg.result_pairs(got, n_rows)) == case["digest"]


@pytest.mark.parametrize("prune,infer", [(False, False), (True, False), (False, True)])
def test_bitvecs_route_matches_oracle(pkg, prune, infer):
    import torch

    syn = pkg.synthetic
    t = syn.plain_small(n_rows=20_000, n_items=300, seed=5)
    bv, col_to_item = bitvecs_of(t.indptr, t.items, t.n_rows)
    dev = torch.from_numpy(bv.view(np.int64)).cuda().view(torch.uint64)
    before = dev.clone()
    got = pkg.apriori(bitvecs=(dev, col_to_item, t.n_rows), min_support=0.005, prune_equal_support=prune,
                      use_generator_pruning=infer, warn_complexity=False)
    ref = miner.mine_bitvecs(bv, t.n_rows, 0.005, prune_equal_support=prune, use_generator_pruning=infer)
    items = np.array([col_to_item[c] for c in range(bv.shape[0])])
    assert pkg.result_pairs(got, t.n_rows) == miner.canonical(ref.levels, items)
    assert torch.equal(dev, before), "the caller's bitvectors must never be written"


def test_dense_bernoulli_matches_oracle(pkg):
    """A dense workload with wide prefix groups (several 64-suffix tiles per group)."""
    import torch

    syn = pkg.synthetic
    p = syn.dense_k2_probs(300, seed=2) * 3
    bv = syn.bernoulli_bitvecs(syn.bernoulli_thresholds(np.minimum(p, 0.9)), 6_000, seed=3)
    dev = torch.from_numpy(bv.view(np.int64)).cuda().view(torch.uint64)
    col_to_item = {c: c for c in range(bv.shape[0])}
    got = pkg.apriori(bitvecs=(dev, col_to_item, 6_000), min_support=0.02, max_length=3, warn_complexity=False)
    ref = miner.mine_bitvecs(bv, 6_000, 0.02, 3)
    assert pkg.result_pairs(got, 6_000) == miner.canonical(ref.levels)


def test_uint64_ids_near_2_63_are_kept(pkg):
    """UInt64 item ids beyond Int64 stay UInt64 in the result (core/result.py:30-54)."""
    base = (1 << 63) - 3
    rows = [[base, base + 1, base + 5], [base, base + 5], [base + 1, base + 5], [base, base + 1, base + 5]]
    got = pkg.apriori(rows, min_support=0.5, use_gpu=True, warn_complexity=False)
    pairs = dict(pkg.result_pairs(got, 4))
    assert pairs[(base, base + 5)] == 3
    assert pairs[(base, base + 1, base + 5)] == 2
    if isinstance(got, pkg.ItemsetFrame):
        assert got.item_dtype == np.uint64


def test_edge_inputs(pkg):
    assert len(pkg.result_pairs(pkg.apriori([], min_support=0.5, use_gpu=True), 1)) == 0
    one = [[4, 2, 2, 9]]
    pairs = pkg.result_pairs(pkg.apriori(one, min_support=1.0, use_gpu=True), 1)
    assert pairs == [((2,), 1), ((4,), 1), ((9,), 1), ((2, 4), 1), ((2, 9), 1), ((4, 9), 1), ((2, 4, 9), 1)]
    got = pkg.apriori(one, min_support=0.0, max_length=1, use_gpu=True)
    assert pkg.result_pairs(got, 1) == [((2,), 1), ((4,), 1), ((9,), 1)]
    # An item in every row is not free: the free-set prune drops it and everything above it.
    rows = [[1, 2], [1, 3], [1, 2, 3], [1]]
    got = pkg.apriori(rows, min_support=0.25, use_gpu=True, prune_equal_support=True)
    assert pkg.result_pairs(got, 4) == [((2,), 2), ((3,), 2), ((2, 3), 1)]


def test_validation_errors(pkg):
    import torch

    dev = torch.zeros((3, 2), dtype=torch.uint64, device="cuda")
    with pytest.raises(ValueError, match="ceil"):
        pkg.apriori(bitvecs=(dev, {0: 1, 1: 2, 2: 3}, 200))
    with pytest.raises(ValueError, match="col_to_item"):
        pkg.apriori(bitvecs=(dev, {0: 1}, 100))
    with pytest.raises(ValueError, match="uint64"):
        pkg.apriori(bitvecs=(dev.view(torch.int64), {0: 1, 1: 2, 2: 3}, 100))
    with pytest.raises(ValueError, match="both"):
        pkg.apriori([[1]], bitvecs=(dev, {0: 1, 1: 2, 2: 3}, 100))
    with pytest.raises(ValueError, match="n_transactions"):
        pkg.apriori(bitvecs=(torch.zeros((1, 1), dtype=torch.uint64, device="cuda"), {0: 1}, 1 << 31))


def test_autotuner_caches_its_choice(pkg, golden_cases, engines):
    """A tuned engine counts each new level shape under every setting once, then reuses the winner."""
    eng = engines["tuned"]
    case = golden_cases["implication_plain"]
    indptr, items, n_rows = case_input(pkg, case)
    for _ in range(2):
        got = pkg.apriori(table_of(indptr, items, n_rows), min_support=case["min_support"], use_gpu=True,
                          engine=eng, warn_complexity=False)
        assert digest_pairs(pkg.result_pairs(got, n_rows)) == case["digest"]
    tuner = eng.autotuner
    assert tuner.cache
    per_key = {}
    for t in tuner.trials:
        per_key[t["key"]] = per_key.get(t["key"], 0) + 1
    assert all(n == len(tuner.settings("tensor")) for n in per_key.values())


def test_level_callback_and_profile(pkg):
    calls = []
    df, session = pkg.apriori([[1, 2, 3], [2, 3, 4], [1, 3, 5], [2, 3]], min_support=0.25, use_gpu=True,
                              level_callback=lambda *a: calls.append(a), profile=True)
    assert [c[0] for c in calls] == [1, 2, 3]
    assert [c[2] for c in calls] == [5, 7, 3]
    assert [p.name for p in session.phases] == ["k1", "k2", "k3"]


def test_row_wise_k3_is_used_and_exact(pkg, golden_cases):
    """The transactions route with the K=3 crossover forced: level 3 is counted row-wise and every level
    equals the bitvector route's."""
    from importlib import import_module

    import torch

    engm = import_module(pkg.__name__ + ".engine")
    api = import_module(pkg.__name__ + ".api")
    case = golden_cases["deep_sparse_small"]
    indptr, items, n_rows = case_input(pkg, case)
    n_cols = int(items.max()) + 1
    bv, rows = api.build_device_bitvecs(indptr, items.astype(np.int32), n_cols, n_rows, keep_rows=True)
    e = _rows_engine(engm.Engine(), k3=True)
    got = e.mine(bv.view(torch.uint64), n_rows, case["min_support"], max_length=case["max_length"], rows=rows)
    assert len(got.stats) >= 3 and got.stats[2].row_wise
    ref = engm.Engine().mine(bv.view(torch.uint64), n_rows, case["min_support"], max_length=case["max_length"])
    assert len(got.levels) == len(ref.levels)
    for a, b in zip(got.levels, ref.levels):
        assert torch.equal(a.rows, b.rows) and torch.equal(a.counts, b.counts)


@pytest.mark.parametrize("name", ["dense_k2_small", "implication_infer", "deep_sparse_small"])
def test_tensor_engine_past_the_exact_row_limit(pkg, golden_cases, monkeypatch, name):
    """Groups over the Gram's exact row limit (2^24 prefix rows; lowered here to 100) and a K=2 level over more
    rows than it count on the CUDA cores within the tensor engine, with the same results."""
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    monkeypatch.setattr(engm, "TC_MAX_ROWS", 100)
    case = golden_cases[name]
    indptr, items, n_rows = case_input(pkg, case)
    got = pkg.apriori(table_of(indptr, items, n_rows), min_support=case["min_support"], max_length=case["max_length"],
                      use_gpu=True, prune_equal_support=case["prune_equal_support"],
                      use_generator_pruning=case["use_generator_pruning"], engine=engm.Engine(method="tensor"),
                      warn_complexity=False)
    assert digest_pairs(pkg.result_pairs(got, n_rows)) == case["digest"]


def test_memory_guards_raise_instead_of_returning_a_partial_lattice(pkg):
    """max_vram_gb / max_ram_gb below what the mine holds: MemoryError after the first counted level."""
    syn = pkg.synthetic
    t = syn.plain_small(n_rows=20_000, n_items=300, seed=5)
    with pytest.raises(MemoryError, match="VRAM"):
        pkg.apriori(table_of(t.indptr, t.items, t.n_rows), min_support=0.005, use_gpu=True, max_vram_gb=1e-9,
                    warn_complexity=False)
    with pytest.raises(MemoryError, match="RAM"):
        pkg.apriori(table_of(t.indptr, t.items, t.n_rows), min_support=0.005, use_gpu=True, max_ram_gb=1e-9,
                    warn_complexity=False)
    got = pkg.apriori(table_of(t.indptr, t.items, t.n_rows), min_support=0.005, use_gpu=True, warn_complexity=False)
    assert len(got) > 0


def test_string_and_float_items_mine_like_their_integer_codes(pkg):
    """Non-integer items: the same itemsets and supports as the integer ids they code to, with the items
    themselves in the result (strings as strings, floats as float64)."""
    syn = pkg.synthetic
    t = syn.plain_small(n_rows=20_000, n_items=300, seed=5)
    want = pkg.result_pairs(pkg.apriori(table_of(t.indptr, t.items, t.n_rows), min_support=0.005, use_gpu=True,
                                        warn_complexity=False), t.n_rows)
    names = np.array([f"item-{i:04d}" for i in range(int(t.items.max()) + 1)])
    rows = [list(names[t.items[t.indptr[r]:t.indptr[r + 1]]]) for r in range(t.n_rows)]
    got = pkg.result_pairs(pkg.apriori(rows, min_support=0.005, use_gpu=True, warn_complexity=False), t.n_rows)
    assert sorted(got) == sorted((tuple(names[i] for i in s), c) for s, c in want)
    floats = [[float(x) + 0.5 for x in t.items[t.indptr[r]:t.indptr[r + 1]]] for r in range(t.n_rows)]
    got_f = pkg.result_pairs(pkg.apriori(floats, min_support=0.005, use_gpu=True, warn_complexity=False), t.n_rows)
    assert sorted(got_f) == sorted((tuple(i + 0.5 for i in s), c) for s, c in want)


@pytest.mark.parametrize("name", ["plain_small_infer", "deep_sparse_small", "implication_infer"])
def test_deduction_bounds_settle_candidates_and_change_nothing(pkg, golden_cases, name):
    """Under generator pruning the deduction bounds (depth <= 3) settle candidates the subset test leaves
    (more INFER or SKIP classes), and the result is the golden one with and without them."""
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    case = golden_cases[name]
    indptr, items, n_rows = case_input(pkg, case)
    settled = {}
    for bounds in (False, True):
        eng = engm.Engine(deduction_bounds=bounds)
        eng.class_stats = True
        got = pkg.apriori(table_of(indptr, items, n_rows), min_support=case["min_support"],
                          max_length=case["max_length"], use_gpu=True, use_generator_pruning=True, engine=eng,
                          warn_complexity=False, level_callback=lambda *a: None)
        ref, col_items = miner.mine_transactions(indptr, items, n_rows, case["min_support"], case["max_length"],
                                                 use_generator_pruning=True)
        assert pkg.result_pairs(got, n_rows) == miner.canonical(ref.levels, col_items)
        settled[bounds] = sum(s.n_inferred + s.n_skipped for s in eng_stats(got, eng))
    assert settled[True] >= settled[False]


def eng_stats(result, eng):
    """The level stats of the engine's last mine (recorded by apriori's profile session)."""
    return eng.last_stats


def test_deduction_bounds_skip_a_candidate_inference_cannot_settle(pkg):
    """100 rows, each holding at least one of a, b, c: 5 x {a,b,c}, 30 x {a,b}, 30 x {a,c}, 35 x {b,c}. Every
    subset of {a,b,c} is frequent and free at min_count 10, so inference leaves it; the depth-3 upper bound
    s(bc)+s(ac)+s(ab) - s(c)-s(b)-s(a) + N = 40+35+35 - 70-70-65 + 100 = 5 (= s(abc), as every row holds one
    of the three) is below 10, so the bounds skip it without counting; the result stays the oracle's."""
    import torch
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    rows = [[0, 1, 2]] * 5 + [[0, 1]] * 30 + [[0, 2]] * 30 + [[1, 2]] * 35
    indptr, items, n_rows = csr_of_rows(rows)
    bv, _ = bitvecs_of(indptr, items, n_rows)
    dev = torch.from_numpy(bv.view(np.int64)).cuda()
    ref = miner.mine_bitvecs(bv, n_rows, 0.1, None, use_generator_pruning=True)
    skipped = {}
    for bounds in (False, True):
        eng = engm.Engine(deduction_bounds=bounds)
        eng.class_stats = True
        out = eng.mine(dev, n_rows, 0.1, None, use_generator_pruning=True)
        assert miner.canonical([(c, n) for c, n in out.host_levels()]) == miner.canonical(ref.levels)
        skipped[bounds] = sum(st.n_skipped for st in out.stats)
    assert skipped == {False: 0, True: 1}


def test_page_locked_results_never_alias_live_ones(pkg, monkeypatch):
    """Results copied back through the page-locked pool: a later call never writes into the buffers of a result
    still alive, and a dropped result's buffer is used again."""
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    monkeypatch.setattr(engm, "PINNED_RESULT_BYTES", 0)
    syn = pkg.synthetic
    t1 = syn.plain_small(n_rows=5_000, n_items=200, seed=11)
    t2 = syn.plain_small(n_rows=7_000, n_items=300, seed=12)
    a = pkg.apriori(table_of(t1.indptr, t1.items, t1.n_rows), min_support=0.01, use_gpu=True, warn_complexity=False)
    pairs_a = pkg.result_pairs(a, t1.n_rows)
    b = pkg.apriori(table_of(t2.indptr, t2.items, t2.n_rows), min_support=0.01, use_gpu=True, warn_complexity=False)
    assert pkg.result_pairs(a, t1.n_rows) == pairs_a
    ref, items = miner.mine_transactions(t2.indptr, t2.items, t2.n_rows, 0.01)
    assert pkg.result_pairs(b, t2.n_rows) == miner.canonical(ref.levels, items)
    n_buffers = len(engm._PINNED.entries)
    del a
    c = pkg.apriori(table_of(t1.indptr, t1.items, t1.n_rows), min_support=0.01, use_gpu=True, warn_complexity=False)
    assert pkg.result_pairs(c, t1.n_rows) == pairs_a
    assert len(engm._PINNED.entries) == n_buffers  # the dropped result's buffer served the new one
