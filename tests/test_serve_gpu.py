"""The continuous-batching server: every result is the same alone and in the mix, and exact.

Requests over three resident datasets are submitted together so that several
run at once on separate streams; each result must equal the same request
mined alone on a fresh engine, and the CPU oracle's result. Tolerance: none
(integer counts).
"""

from __future__ import annotations

from importlib import import_module

import numpy as np
import pytest

from oracle import miner

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(pkg):
    serve = import_module(pkg.__name__ + ".serve")
    syn = pkg.synthetic
    raw = [syn.plain_small(n_rows=n, n_items=m, seed=s) for n, m, s in ((8_000, 200, 1), (20_000, 600, 2), (3_000, 90, 3))]
    datasets = [serve.dataset_from_transactions(t.indptr, t.items) for t in raw]
    return serve, raw, datasets


def _canon(levels):
    return miner.canonical([(np.asarray(s), np.asarray(c)) for s, c in levels])


def test_results_alone_equal_results_in_the_mix(pkg, served):
    serve, raw, datasets = served
    engm = import_module(pkg.__name__ + ".engine")
    reqs = [(d, s, ml) for d in range(3) for s, ml in ((0.01, 3), (0.02, None), (0.005, 4))]
    with serve.Server(datasets, slots=4) as server:
        futs = [server.submit(d, s, ml) for d, s, ml in reqs]
        mixed = [f.result(timeout=300) for f in futs]
        stats = server.stats()
    assert stats["requests"] == len(reqs) and stats["p99_s"] >= stats["p50_s"] > 0
    # Requests on the same dataset with thresholds within 2x share one mine.
    assert any(r.batch > 1 for r in mixed) and stats["mines"] < len(reqs)
    for (d, s, ml), res in zip(reqs, mixed):
        ds = datasets[d]
        alone = engm.Engine(chunk_cands=1 << 24, proj_bytes=1 << 30).mine(ds.bitvecs, ds.n_rows, s, ml)
        alone_levels = [(ds.items[c], n) for c, n in alone.host_levels()]
        assert _canon(res.levels) == _canon(alone_levels), (d, s, ml)
        t = raw[d]
        ref, items = miner.mine_transactions(t.indptr, t.items, t.n_rows, s, ml)
        assert _canon(res.levels) == miner.canonical(ref.levels, items), (d, s, ml)


def test_admission_and_failures(pkg, served):
    serve, _, datasets = served
    with serve.Server(datasets, slots=2, hbm_budget=1 << 20) as server:
        fut = server.submit(1, 0.001, None)
        with pytest.raises(MemoryError):
            fut.result(timeout=60)
    # A dataset whose row count disagrees with its bitvectors fails inside the worker;
    # the server reports it on that request's future and keeps serving the others.
    d0 = datasets[0]
    broken = serve.Dataset(d0.bitvecs, d0.items, d0.n_rows * 100, d0.col_counts)
    with serve.Server(datasets + [broken], slots=2) as server:
        bad = server.submit(3, 0.01, None)
        ok = server.submit(2, 0.05, 2)
        with pytest.raises(ValueError, match="words per column"):
            bad.result(timeout=120)
        assert ok.result(timeout=120).levels


def test_replay_reports_latency(pkg, served):
    serve, _, datasets = served
    syn = pkg.synthetic
    reqs = [r for r in syn.serving_requests(24, mean_gap_s=0.005, seed=7)]
    reqs = [syn.Request(r.dataset % 3, r.min_support * 2, min(r.max_length, 4), r.arrival_s) for r in reqs]
    with serve.Server(datasets, slots=4) as server:
        futs = serve.replay(server, reqs)
        for f in futs:
            f.result(timeout=300)
        st = server.stats()
    assert st["requests"] == 24
    assert st["p99_s"] >= st["p50_s"]


def test_merged_and_unmerged_serving_agree(pkg, served):
    """merge_ratio=1 (every request mined on its own) and the default merging give identical results."""
    serve, _, datasets = served
    reqs = [(1, s, ml) for s, ml in ((0.01, None), (0.012, 3), (0.015, 2), (0.02, None))]
    out = {}
    for ratio in (1.0, 4.0):
        with serve.Server(datasets, slots=1, merge_ratio=ratio) as server:
            futs = [server.submit(d, s, ml) for d, s, ml in reqs]
            out[ratio] = [f.result(timeout=300) for f in futs]
    assert all(r.batch == 1 for r in out[1.0])
    for a, b in zip(out[1.0], out[4.0]):
        assert _canon(a.levels) == _canon(b.levels)
