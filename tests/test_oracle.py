"""The CPU oracle against the reference CPU route's golden results (tests/golden/cases.json)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import miner
from tests.conftest import case_input

CASES = [c["name"] for c in json.loads((Path(__file__).parent / "golden" / "cases.json").read_text())["cases"]]
SLOW = {"wide_vocab_small"}


@pytest.mark.parametrize("name", [n for n in CASES if n not in SLOW])
def test_oracle_matches_reference(pkg, golden_cases, name):
    case = golden_cases[name]
    indptr, items, n_rows = case_input(pkg, case)
    res, col_items = miner.mine_transactions(
        indptr, items, n_rows, case["min_support"], case["max_length"],
        prune_equal_support=case["prune_equal_support"], use_generator_pruning=case["use_generator_pruning"],
    )
    assert res.level_sizes() == case["level_sizes"]
    assert miner.digest(res.levels, col_items) == case["digest"]
    if "itemsets" in case:
        want = sorted((tuple(s), c) for s, c in case["itemsets"])
        assert miner.canonical(res.levels, col_items) == sorted(want, key=lambda t: (len(t[0]), t[0]))


@pytest.mark.slow
@pytest.mark.parametrize("name", sorted(SLOW))
def test_oracle_matches_reference_large(pkg, golden_cases, name):
    test_oracle_matches_reference(pkg, golden_cases, name)


def test_min_count_fixture():
    """The exact decimal ceiling (core/result.py:57-79) on the reference's shared min-count table."""
    cases = json.loads((Path(__file__).parent / "golden" / "min_count_cases.json").read_text())["cases"]
    for c in cases:
        assert miner.min_count(c["min_support"], c["n_rows"]) == c["expected"], c


def test_boundary_cone_kept(golden_cases):
    """0.07 x 10,000 -> 700: the itemset at exactly the threshold and its cone are frequent."""
    got = {tuple(s) for s, _ in golden_cases["boundary_cone"]["itemsets"]}
    assert {(0,), (0, 1), (0, 2), (0, 1, 2)} <= got


def test_four_rows_supports(golden_cases):
    """The 4-row fixture: supports 0.5 / 0.75 / 1.0 for 1 / 2 / 3, pairs (1,3) 0.5 and (2,3) 0.75."""
    got = {tuple(s): c / 4 for s, c in golden_cases["four_rows_plain"]["itemsets"]}
    assert got == {(1,): 0.5, (2,): 0.75, (3,): 1.0, (1, 3): 0.5, (2, 3): 0.75}


def test_digest_is_order_free():
    a = [(np.array([[0, 1], [0, 2]], np.int32), np.array([5, 4]))]
    b = [(np.array([[0, 2], [0, 1]], np.int32), np.array([4, 5]))]
    assert miner.digest(a) == miner.digest(b)


def test_cpu_route_matches_the_golden_results(pkg, golden_cases):
    """The restated CPU route (sparse Gram K=2, prefix-group projection Grams K>=3, thread pool) reproduces
    the golden digest of every case, unbounded (the 1M-row wide-vocabulary case is left to the GPU tests for
    time: its route mine alone takes about 20 s here)."""
    from oracle import cpu_route, miner
    from tests.conftest import case_input

    checked = 0
    for case in golden_cases.values():
        if case["name"].startswith("wide_vocab"):
            continue
        indptr, items, n_rows = case_input(pkg, case)
        csr = miner.transaction_csr(indptr, items, n_rows, case["min_support"])
        if csr is None:
            continue
        got = cpu_route.mine(csr.indptr, csr.cols, csr.n_cols, n_rows, case["min_support"], case["max_length"],
                             prune_equal_support=case["prune_equal_support"],
                             use_generator_pruning=case["use_generator_pruning"], workers=3)
        assert got.complete
        assert miner.digest(got.levels, csr.items) == case["digest"], case["name"]
        checked += 1
    assert checked >= 30


def test_cpu_route_budget_stops_early_and_says_so(pkg):
    """With a time budget that has already run out the route counts K=1 only and reports itself incomplete."""
    from oracle import cpu_route, miner

    t = pkg.synthetic.plain_small(n_rows=20_000, seed=1)
    csr = miner.transaction_csr(t.indptr, t.items, t.n_rows, 0.01)
    r = cpu_route.mine(csr.indptr, csr.cols, csr.n_cols, t.n_rows, 0.01, None, workers=2, budget_s=0.0)
    assert not r.complete
    assert r.counted[0]["k"] == 1 and r.counted[1]["counted"] == 0
