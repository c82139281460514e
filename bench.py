"""Benchmark: exact Apriori mining of the dense K=2 stress workload on one GB300.

Workload (default ``dense_k2``): 2,000,000 transactions x 4,096 items, item
i present independently with probability p_i ~ Beta(2, 30) (hash-defined
bits, generated on the device), min_support 0.002, max_length 3. One step is
one complete ``mine()`` of that workload: K=1, the ~8.4M pair candidates and
the ~4.4e9 triple candidates, every survivor compacted into lexsorted
levels. The bitvectors (1.02 GB) are larger than L2, so no flush is needed
between steps.

Prints ONE JSON line (rank 0):
  value         seconds per mine, batched form (device-resident input)
  exact         the benchmarked result checked: sampled recounts in plain
                PyTorch, subset closure, completeness/absence of random
                extensions, level 1 complete (verify.check_mine)
  plain         the one-launch-per-prefix-group form on the same input
  e2e           seconds per mine through apriori(bitvecs=...) with the
                bitvectors copied from pinned host memory and the itemsets
                copied back inside the timed region
  roofline      the dominant kernel: useful work per launch over its
                CUDA-event time, against the measured peak of its unit (the
                Gram's own MMA rate for the tensor-core kernel)
  cpu_baseline  the reference's CPU route (oracle/cpu_route.py) on every host
                core, on the same input, under a time budget: measured, a
                lower bound when the budget ran out before the mine finished
  workloads     the plain small workload through the transactions route and
                the deep sparse workload (20M rows, generator pruning), each
                with its own check and CPU route beside it
``--impl reference`` runs the reference's CPU route alone on the same
workload, each step one budgeted mine.

Multi-GPU: the path does not shard in this engine (replicas only); under
torchrun every rank mines its own copy and the max over ranks is reported.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

WORKLOADS = {
    "dense_k2": dict(n_items=4096, n_rows=2_000_000, min_support=0.002, max_length=3, seed=0, hash_seed=12345),
    "dense_k2_mid": dict(n_items=2048, n_rows=1_000_000, min_support=0.002, max_length=3, seed=0, hash_seed=12345),
    "dense_k2_small": dict(n_items=1024, n_rows=500_000, min_support=0.002, max_length=3, seed=0, hash_seed=12345),
}


#: DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic byte of a kernel, from one ncu
#: capture of every Gram, projection and transpose launch of the 1M x 2048 dense K=2 workload (four mines:
#: warm-up, timed step, two end-to-end calls):
#:   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none
#:       -k "regex:gram_kernel|project_rows|rows_transpose" python bench.py --workload dense_k2_mid --steps 1
#:       --warmup 1 --no-plain --no-cpu --no-side --no-serial --no-hbm --no-pipeline
#: per mine 15.89 GB against 12.66 GB for the Gram, 21.26 GB against 46.00 GB for the row-major projection
#: (its prefix rows' row words come partly from L2), 0.50 GB against 0.51 GB for the transpose; the roofline's
#: ``traffic`` scales it to the bench's own launches by their algorithmic bytes.
DRAM_PER_ALGORITHMIC_BYTE = {"gram_tc": 15.892 / 12.659, "project_rows": 21.262 / 45.998, "rows_transpose": 0.495 / 0.511}


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        self.device_index = device_index
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(device_index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dense_k2_device(pkg, lib, spec):
    import torch

    syn = pkg.synthetic
    p = syn.dense_k2_probs(spec["n_items"], seed=spec["seed"])
    thr = torch.from_numpy(syn.bernoulli_thresholds(p).view(np.int64)).cuda()
    n_rows = spec["n_rows"]
    ld = (n_rows + 63) // 64
    bv = torch.empty((spec["n_items"], ld), dtype=torch.int64, device="cuda")
    st = lib.etm_synth_bernoulli(thr.data_ptr(), spec["n_items"], n_rows, spec["hash_seed"], bv.data_ptr(), ld,
                                 torch.cuda.current_stream().cuda_stream)
    if st != 0:
        raise RuntimeError(lib.etm_last_error().decode())
    torch.cuda.synchronize()
    return bv.view(torch.uint64)


#: Candidates per level of each workload (K=1 columns, K=2 pairs, K=3 prefix-group pairs), as the engine
#: enumerates them; the engine arm asserts its own counts against these on every run.
LEVEL_CANDIDATES = {
    "dense_k2": [4096, 8_345_655, 5_155_139_504],
    "dense_k2_mid": None,
    "dense_k2_small": [1024, 522_753, 73_706_695],
}


_MP_SPEC = None


def _mp_init(spec) -> None:
    global _MP_SPEC
    _MP_SPEC = spec


def _mp_item_rows(items) -> list:
    """Row ids holding each listed item of the hash-defined Bernoulli workload (host restatement of
    etm_synth_bernoulli), in chunks of 2^20 rows."""
    import __graft_entry__ as g

    syn = g.package().synthetic
    thr, n_rows, seed = _MP_SPEC
    out = []
    for i in items:
        parts = []
        for r0 in range(0, n_rows, 1 << 20):
            rows = np.arange(r0, min(n_rows, r0 + (1 << 20)), dtype=np.uint64)
            h = syn.bit_hash(seed, np.full(len(rows), i, dtype=np.uint64), rows)
            parts.append(np.flatnonzero(h < thr[i]).astype(np.int32) + r0)
        out.append(np.concatenate(parts))
    return out


def dense_k2_host_csr(pkg, spec, workers: int):
    """The dense K=2 workload as the CPU route's input: the frequent-column CSR of the transactions (built on
    the host cores from the same hash-defined bits the device generates), and the seconds it took."""
    import multiprocessing as mp

    from oracle import cpu_route

    t0 = time.perf_counter()
    syn = pkg.synthetic
    thr = syn.bernoulli_thresholds(syn.dense_k2_probs(spec["n_items"], seed=spec["seed"]))
    items = np.array_split(np.arange(spec["n_items"]), max(1, 4 * workers))
    with mp.get_context("spawn").Pool(workers, initializer=_mp_init,
                                      initargs=((thr, spec["n_rows"], spec["hash_seed"]),)) as pool:
        rows = [r for part in pool.map(_mp_item_rows, items, chunksize=1) for r in part]
    indptr, cols = cpu_route.csr_from_column_rows(rows, spec["n_rows"])
    del rows
    fp, fc, kept = cpu_route.frequent_csr(indptr, cols, spec["n_items"], spec["n_rows"], spec["min_support"])
    return (fp, fc, len(kept)), time.perf_counter() - t0


def cpu_route_timed(csr, n_rows: int, min_support: float, max_length, budget_s: float | None, workers: int,
                    **flags) -> dict:
    """One mine of the reference's CPU route (oracle/cpu_route.py) on the host cores: measured seconds, and
    whether it finished within ``budget_s`` (if not, the seconds are a lower bound of the whole mine's)."""
    from oracle import cpu_route

    indptr, cols, n_cols = csr
    r = cpu_route.mine(indptr, cols, n_cols, n_rows, min_support, max_length, workers=workers, budget_s=budget_s,
                       **flags)
    return {"value": r.seconds, "complete": r.complete, "counted": r.counted, "itemsets": sum(len(s) for s, _ in r.levels),
            "levels": r.levels}


def cpu_model() -> str:
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


def _baseline_entry(run: dict, cores: int, what: str) -> dict:
    return {"value": run["value"], "unit": "s", "cores": cores, "kind": "port",
            "lower_bound": not run["complete"], "counted": run["counted"], "cpu": cpu_model(),
            "sample": what + (" (the whole mine)" if run["complete"] else
                              " until the time budget ran out: the value is the measured time of the part counted "
                              "(see counted), a lower bound of the whole mine's time, not an extrapolation")}


def max_over_ranks(value: float, dist=None, device: str = "cuda") -> float:
    """The largest of every rank's ``value`` (the replicas' slowest mine); ``value`` itself without a process
    group."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


ROUTE_SAMPLE = ("oracle/cpu_route.py mine: the reference's CPU route (scipy Gram column blocks for K=2, prefix-group "
                "projection Grams for K>=3, core/cpu_miner.py:332-378, 727-791, 1066-1161) over a thread pool of "
                "every host core")


def run_reference(args, spec) -> None:
    """The reference's CPU route on the same workload, on every host core: each timed step one mine under a
    time budget (the whole run stays within a few minutes)."""
    pkg = _pkg()
    workers = max(1, os.cpu_count() or 1)
    csr, build_s = dense_k2_host_csr(pkg, spec, workers)
    budget = args.ref_budget if args.ref_budget else max(20.0, min(90.0, 180.0 / max(1, args.steps)))
    runs = [cpu_route_timed(csr, spec["n_rows"], spec["min_support"], spec["max_length"], budget, workers)
            for _ in range(max(1, args.steps))]
    value = statistics.median(r["value"] for r in runs)
    base = _baseline_entry(runs[0], workers, ROUTE_SAMPLE + f", {budget:.0f} s budget per step")
    base["value"] = value
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
        "steps": len(runs), "warmup": 0, "ms_per_step": value * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (hash-defined Bernoulli bits, host)",
        "config": {"workload": args.workload, **spec}, "lower_bound": not runs[0]["complete"],
        "input_build_s": build_s, "cpu_baseline": base,
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


TX_METRIC = "apriori(transactions) seconds, plain small (60K x 1,000, s=0.01), exact counts"
#: Workloads mined through the transactions route (host CSR in, result frame out).
TX_WORKLOADS = {
    "plain_small_tx": dict(gen="plain_small", n_rows=60_000, n_items=1_000, min_support=0.01, max_length=None, seed=0),
}


def _tx_cpu_mine(t, spec):
    """The CPU route of a transactions workload on every host core: the frequent-item CSR, then the level
    loop (both timed): (seconds, canonical result, cores)."""
    from oracle import cpu_route, miner

    workers = max(1, os.cpu_count() or 1)
    t0 = time.perf_counter()
    csr = miner.transaction_csr(t.indptr, t.items, t.n_rows, spec["min_support"])
    r = cpu_route.mine(csr.indptr, csr.cols, csr.n_cols, t.n_rows, spec["min_support"], spec["max_length"],
                       workers=workers)
    return time.perf_counter() - t0, miner.canonical(r.levels, csr.items), workers


def transactions_line(pkg, name: str, steps: int, warmup: int, with_cpu: bool = True) -> dict:
    """The transactions route on a workload of TX_WORKLOADS (the plain small one: 60K rows x 1,000
    Zipf(1.1) items, s=0.01): seconds per ``apriori(transactions, use_gpu=True)`` call (transaction CSR on the
    host in, result frame out), the kernels it ran, exactness against the CPU route's own result, and the CPU
    route's whole mine of the same input timed beside it (small enough to run in full)."""
    import torch

    spec = TX_WORKLOADS[name]
    t = getattr(pkg.synthetic, spec["gen"])(seed=spec["seed"])
    n_rows = t.n_rows
    pkg.build_library()
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine()
    eng.profile_kernels = True
    levels = []

    def call():
        levels.clear()
        return pkg.apriori(t, min_support=spec["min_support"], max_length=spec["max_length"], use_gpu=True,
                           engine=eng, warn_complexity=False,
                           level_callback=lambda k, nc, nf, ms: levels.append({"k": k, "candidates": nc,
                                                                               "frequent": nf}))

    for _ in range(max(1, warmup)):
        df = call()
    torch.cuda.synchronize()
    eng.reset_kernel_times()
    launches0 = eng.launches
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    t0 = time.perf_counter()
    for _ in range(steps):
        df = call()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    clk = clocks.stop()
    kern = eng.kernel_report()
    got = pkg.result_pairs(df, n_rows)
    n_sets = len(got)
    n_vals = sum(len(s) for s, _ in got)
    line = {
        "metric": TX_METRIC, "value": dt, "unit": "s", "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded plain_small generator, host CSR)",
        "config": {"workload": name, **spec, "route": "transactions"},
        "levels": list(levels), "itemsets": n_sets,
        "e2e": {"value": dt, "unit": "s", "h2d_bytes_per_step": int(t.indptr.nbytes + t.items.nbytes),
                "d2h_bytes_per_step": 8 * n_vals + 16 * n_sets + 8},
        "kernels": kern, "gpu_launches": (eng.launches - launches0) // steps, "clocks": clk,
    }
    if with_cpu:
        cpu_s, want, workers = _tx_cpu_mine(t, spec)
        line["exact"] = got == want
        line["cpu_baseline"] = {"value": cpu_s, "unit": "s", "cores": workers, "kind": "port", "lower_bound": False,
                                "cpu": cpu_model(),
                                "sample": "oracle/miner.py transaction_csr + " + ROUTE_SAMPLE + " (the whole mine)"}
    return line


def run_transactions(args) -> None:
    spec = TX_WORKLOADS[args.workload]
    pkg = _pkg()
    if args.impl == "reference":
        t = getattr(pkg.synthetic, spec["gen"])(seed=spec["seed"])
        cpu_s, _, workers = _tx_cpu_mine(t, spec)
        base = {"value": cpu_s, "unit": "s", "cores": workers, "kind": "port", "lower_bound": False,
                "cpu": cpu_model(), "sample": "oracle/miner.py transaction_csr + " + ROUTE_SAMPLE + " (the whole mine)"}
        print(json.dumps({"impl": "reference", "metric": TX_METRIC, "value": cpu_s, "unit": "s", "n_gpus": args.gpus,
                          "steps": 1, "warmup": 0, "ms_per_step": cpu_s * 1e3, "higher_is_better": False,
                          "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
                          "config": {"workload": args.workload, **spec}, "cpu_baseline": base,
                          "e2e": {"value": cpu_s, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return
    print(json.dumps(transactions_line(pkg, args.workload, args.steps, args.warmup)), flush=True)


#: The deep sparse workload: 20M transactions over 2,000 items from 500 planted patterns (hash-defined,
#: generated on the device), min_support 0.005, max_length 16, generator pruning.
DEEP_SPARSE = dict(n_rows=20_000_000, n_items=2_000, min_support=0.005, max_length=16, use_generator_pruning=True,
                   pattern_seed=0, hash_seed=777)


def device_bitvecs_to_host_csr(bv, n_rows: int, chunk_cols: int = 64):
    """The row-major CSR (indptr int64, column ids int32) of device bitvectors, built on the device (bits
    unpacked per column chunk, entries sorted by row) and copied to the host: the CPU route's input."""
    import torch

    n_cols = bv.shape[0]
    b = bv.view(torch.int64)
    shifts = torch.arange(64, device=b.device, dtype=torch.int64)
    keys = []
    for c0 in range(0, n_cols, chunk_cols):
        x = b[c0:c0 + chunk_cols]
        bits = ((x[:, :, None] >> shifts) & 1).view(x.shape[0], -1)[:, :n_rows]
        col, row = torch.nonzero(bits, as_tuple=True)
        keys.append(row * n_cols + (col + c0))
        del bits
    k = torch.sort(torch.cat(keys)).values
    rows, cols = k // n_cols, (k % n_cols).to(torch.int32)
    indptr = torch.zeros(n_rows + 1, dtype=torch.int64, device=b.device)
    indptr[1:] = torch.cumsum(torch.bincount(rows, minlength=n_rows), 0)
    return indptr.cpu().numpy(), cols.cpu().numpy()


def deep_sparse_line(pkg, lib, steps: int, warmup: int, with_cpu: bool, cpu_budget_s: float = 40.0) -> dict:
    """The deep sparse workload mined on the device (bitvectors resident), checked by ``verify.check_mine``,
    with the CPU route on the same input under a time budget beside it."""
    import torch
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    verm = import_module(pkg.__name__ + ".verify")
    spec = DEEP_SPARSE
    syn = pkg.synthetic
    n_rows = spec["n_rows"]
    ps = syn.pattern_spec(n_items=spec["n_items"], seed=spec["pattern_seed"], hash_seed=spec["hash_seed"])
    bv = syn.patterns_bitvecs_device(lib, ps, n_rows)
    eng = engm.Engine()

    def one():
        return eng.mine(bv, n_rows, spec["min_support"], spec["max_length"], use_generator_pruning=True)

    for _ in range(max(1, warmup)):
        out = one()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = eng.launches
    start.record()
    for _ in range(steps):
        out = one()
    end.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / steps
    rep = verm.check_mine(out, bv, n_rows, generators=True, max_length=spec["max_length"], sample=10_000)
    # End to end through apriori(bitvecs=): the 5 GB of bitvectors copied in from pinned host memory and the
    # result frame copied back, every step.
    host = torch.empty(bv.shape, dtype=torch.int64, pin_memory=True)
    host.copy_(bv.view(torch.int64))
    dev = torch.empty_like(bv.view(torch.int64))
    col_to_item = {c: c for c in range(bv.shape[0])}
    e2e_ms = []
    for i in range(steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev.copy_(host, non_blocking=True)
        df = pkg.apriori(bitvecs=(dev.view(torch.uint64), col_to_item, n_rows), min_support=spec["min_support"],
                         max_length=spec["max_length"], use_generator_pruning=True, engine=eng, warn_complexity=False)
        torch.cuda.synchronize()
        if i > 1:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    n_sets = len(df)
    del df, host, dev
    line = {"workload": "deep_sparse", "config": {**spec, "rows_generated_on": "device (etm_synth_patterns)"},
            "metric": "mine() seconds, bitvectors resident", "value": ms / 1e3, "unit": "s", "steps": steps,
            "e2e": {"value": statistics.median(e2e_ms) / 1e3, "unit": "s", "steps_ms": [round(x, 2) for x in e2e_ms],
                    "h2d_bytes_per_step": int(bv.numel() * 8),
                    "d2h_bytes_per_step": int(8 * sum(lv.n * lv.k for lv in out.levels) + 8 * len(out.level1_cols)
                                              + 16 * out.n_itemsets() + 8),
                    "itemsets": n_sets},
            "levels": [{"k": s.k, "candidates": s.n_candidates, "frequent": s.n_frequent} for s in out.stats],
            "itemsets": out.n_itemsets(), "gpu_launches": (eng.launches - launches0) // steps,
            "exact": {"sampled": rep["sampled"], "mismatches": rep["mismatches"],
                      "extensions_checked": rep["extensions_checked"], "level1_complete": rep["level1_complete"]}}
    if with_cpu:
        t0 = time.perf_counter()
        indptr, cols = device_bitvecs_to_host_csr(bv, n_rows)
        from oracle import cpu_route

        csr = cpu_route.frequent_csr(indptr, cols, spec["n_items"], n_rows, spec["min_support"])
        build_s = time.perf_counter() - t0
        workers = max(1, os.cpu_count() or 1)
        run = cpu_route_timed((csr[0], csr[1], len(csr[2])), n_rows, spec["min_support"], spec["max_length"],
                              cpu_budget_s, workers, use_generator_pruning=True)
        line["cpu_baseline"] = _baseline_entry(run, workers, ROUTE_SAMPLE + f", {cpu_budget_s:.0f} s budget")
        line["cpu_baseline"]["input_build_s"] = build_s
        if run["complete"]:
            from oracle import miner

            got = [(c, n) for c, n in out.host_levels()]
            line["cpu_baseline"]["equal_to_engine"] = miner.canonical(got) == miner.canonical(
                [(csr[2][s], c) for s, c in run["levels"]])
        del run
    del bv
    torch.cuda.empty_cache()
    return line


TILE_PAIR_WORDS = 64 * 64  # pair counts a 64 x 64 tile-pair updates per word


def hbm_kernel_rooflines(pkg, lib, n_rows: int = 20_000_000, reps: int = 3) -> list[dict]:
    """The AND+popcount and bitvector kernels on the deep sparse workload's shape (20M rows x 2,000 items,
    planted patterns, generated on the device): per kernel its CUDA-event time (median of ``reps`` after a
    warm-up), algorithmic bytes, GB/s and fraction of the measured HBM copy peak. Inputs (5 GB of
    bitvectors) are larger than L2."""
    import torch
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    syn = pkg.synthetic
    peak = _peaks()["hbm_gbs"]
    st = torch.cuda.current_stream().cuda_stream
    bv = syn.patterns_bitvecs_device(lib, syn.pattern_spec(), n_rows)
    n_cols, ld = bv.shape
    n_words = (n_rows + 63) // 64
    bvi = bv.view(torch.int64)
    # The device CSR of the same rows (the bitvector build's input).
    shifts = torch.arange(64, device="cuda", dtype=torch.int64)
    keys = []
    for c0 in range(0, n_cols, 64):
        bits = ((bvi[c0:c0 + 64][:, :, None] >> shifts) & 1).view(min(64, n_cols - c0), -1)[:, :n_rows]
        col, row = torch.nonzero(bits, as_tuple=True)
        keys.append(row * n_cols + (col + c0))
        del bits
    k = torch.sort(torch.cat(keys)).values
    del keys
    ids = (k % n_cols).to(torch.int32)
    row_ptr = torch.zeros(n_rows + 1, dtype=torch.int64, device="cuda")
    row_ptr[1:] = torch.cumsum(torch.bincount(k // n_cols, minlength=n_rows), 0)
    del k
    nnz = int(ids.numel())
    out_bv = torch.empty_like(bvi)
    counts = torch.empty(n_cols, dtype=torch.int64, device="cuda")
    eng = engm.Engine()
    fbv, ldp = eng.gather(bvi.data_ptr(), ld, np.arange(n_cols), n_words)
    # count_cands: 4,096 random triples of frequent columns as 2-member prefix groups; count_tiles: one group of
    # 128 columns over every row (the K=2 tile kernel on unprojected words).
    rng = np.random.default_rng(0)
    pairs = np.sort(np.stack([rng.choice(n_cols, 3, replace=False) for _ in range(4096)]), axis=1)
    gen_rows = np.concatenate([pairs[:, [0, 1]], pairs[:, [0, 2]]])
    gen_rows = np.unique(gen_rows, axis=0).astype(np.int32)
    gen = engm.Level(torch.from_numpy(gen_rows).cuda(), torch.ones(len(gen_rows), dtype=torch.int32, device="cuda"))
    G, total, grp_first, grp_size, cand_off = eng.groups(gen)
    sizes = grp_size[:G].cpu().numpy().astype(np.int64)
    wg_c, wo_c = eng._work(np.arange(G, dtype=np.int64), sizes * (sizes - 1) // 2)
    cand_counts = torch.empty(max(1, total), dtype=torch.int32, device="cuda")
    m_t = 128
    gen_t = engm.Level(torch.arange(m_t, dtype=torch.int32, device="cuda")[:, None].contiguous(),
                       torch.ones(m_t, dtype=torch.int32, device="cuda"))
    Gt, total_t, gf_t, gs_t, co_t = eng.groups(gen_t)
    nt = (m_t + 63) // 64
    wg_t, wo_t = eng._work(np.zeros(1, np.int64), np.array([nt * (nt + 1) // 2]))
    tile_counts = torch.empty(total_t, dtype=torch.int32, device="cuda")
    n_tp = nt * (nt + 1) // 2
    n_split = int(max(1, min(-(-n_words // 32), (6 * int(lib.etm_device_sm_count())) // n_tp)))
    eng_cols = torch.arange(n_cols, dtype=torch.int32, device="cuda")
    kernels = {
        "build_bitvecs": (lambda: lib.etm_build_bitvecs(row_ptr.data_ptr(), ids.data_ptr(), nnz, None, 0, n_rows,
                                                        n_cols, ld, out_bv.data_ptr(), st),
                          8 * (n_rows + 1) + 4 * nnz + 8 * n_cols * ld, "8(N+1) + 4 nnz read, 8 n_cols W written"),
        "popcount_cols": (lambda: lib.etm_popcount_cols(bvi.data_ptr(), n_cols, n_words, ld, counts.data_ptr(), st),
                          8 * n_cols * n_words, "8 n_cols W read"),
        "gather_cols": (lambda: lib.etm_gather_cols(bvi.data_ptr(), ld, eng_cols.data_ptr(), n_cols, n_words,
                                                    fbv.data_ptr(), ldp, st),
                        16 * n_cols * n_words, "8 n_cols W read + written"),
        "count_cands": (lambda: lib.etm_count_cands(fbv.data_ptr(), ldp, n_words, gen.rows.data_ptr(), 2,
                                                    grp_first.data_ptr(), grp_size.data_ptr(), cand_off.data_ptr(),
                                                    wg_c.data_ptr(), wo_c.data_ptr(), G, 0, None,
                                                    cand_counts.data_ptr(), st),
                        8 * 3 * n_words * total, "8 k W per candidate (k = 3)"),
        "count_tiles": (lambda: (tile_counts.zero_(), lib.etm_count_tiles_split(
                            fbv.data_ptr(), ldp, n_words, gen_t.rows.data_ptr(), 1, gf_t.data_ptr(), gs_t.data_ptr(),
                            co_t.data_ptr(), wg_t.data_ptr(), wo_t.data_ptr(), 1, n_tp, 0, None, n_split,
                            tile_counts.data_ptr(), st))[1],
                        8 * m_t * n_words, "8 m W: each column once (the same-data minimum); word ranges split "
                                           "across CTAs as the engine splits them"),
    }
    out = []
    for name, (fn, nbytes, how) in kernels.items():
        times = []
        for i in range(reps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            if fn() != 0:
                raise RuntimeError(f"{name}: {lib.etm_last_error().decode()}")
            e1.record()
            torch.cuda.synchronize()
            if i:
                times.append(e0.elapsed_time(e1))
        ms = statistics.median(times)
        gbs = nbytes / (ms / 1e3) / 1e9
        out.append({"kernel": name, "ms": round(ms, 3), "algorithmic_bytes": int(nbytes), "bytes": how,
                    "achieved_gbs": round(gbs, 1), "peak_gbs": peak, "frac": round(gbs / peak, 3)})
    # The tile kernel is bound by the popcount pipe (64 x 64 pair counts per staged word pair), so its roofline is
    # the measured AND+popcount issue rate of its inner loop; the HBM fraction above is only its input stream.
    import ctypes

    rate = ctypes.c_double(0.0)
    if lib.etm_popc_rate(1 << 14, ctypes.byref(rate), st) != 0:
        raise RuntimeError(lib.etm_last_error().decode())
    tiles = next(r for r in out if r["kernel"] == "count_tiles")
    useful = m_t * (m_t - 1) // 2 * n_words
    issued = n_tp * TILE_PAIR_WORDS * n_words
    gops = useful / (tiles["ms"] / 1e3) / 1e9
    tiles.update({"bound": "popc", "pair_words": useful, "issued_pair_words": issued,
                  "achieved_gops": round(gops, 1), "popc_peak_gops": round(rate.value, 1),
                  "frac_popc": round(gops / rate.value, 3),
                  "frac_popc_issued": round(issued / (tiles["ms"] / 1e3) / 1e9 / rate.value, 3),
                  "peak_source": "measured: etm_popc_rate (the tile kernel's 4 x 4 AND+popcount block on every SM)"})
    for r in out:
        r.setdefault("bound", "hbm")
    # The outputs agree with each other: K=1 counts of the rebuilt bitvectors equal those of the originals.
    assert torch.equal(out_bv, bvi), "build_bitvecs does not reproduce the generator's bitvectors"
    del bv, bvi, out_bv, fbv, ids, row_ptr
    torch.cuda.empty_cache()
    return out


def run_hbm_kernels(args) -> None:
    pkg = _pkg()
    pkg.build_library()
    lib = pkg.load_library()
    rows = hbm_kernel_rooflines(pkg, lib, n_rows=args.hbm_rows)
    print(json.dumps({"metric": "AND+popcount and bitvector kernels, GB/s against the measured HBM copy peak",
                      "workload": "hbm_kernels", "config": {"rows": args.hbm_rows, "items": 2_000,
                                                            "input": "deep sparse planted patterns, device-generated"},
                      "rooflines": rows}), flush=True)


def run_serving(args) -> None:
    """Serving workload: 256 Poisson-arriving requests over 8 resident datasets, p50/p99 latency."""
    import torch

    from oracle import miner

    pkg = _pkg()
    pkg.build_library()
    from importlib import import_module

    serve = import_module(pkg.__name__ + ".serve")
    engm = import_module(pkg.__name__ + ".engine")
    syn = pkg.synthetic
    t0 = time.perf_counter()
    raw = syn.serving_datasets(seed=0, scale=args.serving_scale)
    datasets = [serve.dataset_from_transactions(t.indptr, t.items) for t, _ in raw]
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    reqs = syn.serving_requests(args.serving_requests, mean_gap_s=0.05, seed=0)
    # Warm-up: one small request per dataset (library load, first launches).
    with serve.Server(datasets, slots=args.slots) as server:
        for f in [server.submit(d, 0.05, 2) for d in range(len(datasets))]:
            f.result()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    with serve.Server(datasets, slots=args.slots) as server:
        t1 = time.perf_counter()
        futs = serve.replay(server, reqs)
        results = [f.result() for f in futs]
        makespan = time.perf_counter() - t1
        st = server.stats()
    # Capacity: the same requests all queued at once (arrival times ignored), merged and one mine each.
    capacity = {}
    for name, ratio in (("merged", 2.0), ("one_mine_per_request", 1.0)):
        with serve.Server(datasets, slots=args.slots, merge_ratio=ratio) as server:
            t2 = time.perf_counter()
            futs_c = [server.submit(r.dataset, r.min_support, r.max_length) for r in reqs]
            for f in futs_c:
                f.result()
            span = time.perf_counter() - t2
            sc = server.stats()
        capacity[name] = {"requests_per_s": len(reqs) / span, "makespan_s": span, "mines": sc["mines"],
                          "p50_s": sc["p50_s"], "p99_s": sc["p99_s"]}
    clk = clocks.stop()
    # Exactness: every request against the same request mined alone (one engine, nothing else on the GPU),
    # and the CPU oracle on the small datasets.
    sample = np.arange(len(reqs))
    alone_ok = oracle_ok = 0
    oracle_n = 0
    alone_eng = engm.Engine(chunk_cands=1 << 24, proj_bytes=1 << 30)
    for i in sample:
        r, res = reqs[i], results[i]
        ds = datasets[r.dataset]
        alone = alone_eng.mine(ds.bitvecs, ds.n_rows, r.min_support, r.max_length)
        a_levels = [(ds.items[c], n) for c, n in alone.host_levels()]
        got = miner.canonical(res.levels)
        alone_ok += int(got == miner.canonical(a_levels))
        if ds.n_rows <= 60_000 and oracle_n < 12:
            t = raw[r.dataset][0]
            ref, items = miner.mine_transactions(t.indptr, t.items, t.n_rows, r.min_support, r.max_length)
            oracle_ok += int(got == miner.canonical(ref.levels, items))
            oracle_n += 1
    line = {
        "metric": "serving p99 latency, 256 Poisson requests (mean gap 50 ms) over 8 resident datasets",
        "value": st["p99_s"], "unit": "s", "n_gpus": 1, "steps": 1, "warmup": len(datasets),
        "ms_per_step": makespan * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic (seeded serving datasets and request stream)",
        "config": {"workload": "serving", "requests": len(reqs), "slots": args.slots, "scale": args.serving_scale,
                   "datasets": [{"rows": ds.n_rows, "items": ds.n_cols} for ds in datasets]},
        "p50_s": st["p50_s"], "p99_s": st["p99_s"], "mean_s": st["mean_s"], "max_s": st["max_s"],
        "queued_p99_s": st["queued_p99_s"], "throughput_rps": len(reqs) / makespan, "makespan_s": makespan,
        "mines": st["mines"], "capacity": capacity,
        "dataset_build_s": build_s,
        "exact": {"alone_equal": f"{alone_ok}/{len(sample)}", "oracle_equal": f"{oracle_ok}/{oracle_n}"},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def _pkg():
    import __graft_entry__ as g

    return g.package()


#: Operand formats of the tensor-core Gram by element code.
OPERANDS = {1: "e4m3 (kind::f8f6f4)", 2: "f16 (kind::f16)", 4: "packed e2m1 (kind::mxf4, unit block scales)"}

METRIC = "mine() seconds, dense K=2 stress (2M x 4096, s=0.002, max_length=3), exact counts, batched form"


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="dense_k2",
                    choices=sorted(WORKLOADS) + sorted(TX_WORKLOADS) + ["serving", "hbm_kernels"])
    ap.add_argument("--slots", type=int, default=4, help="serving: requests on the GPU at once")
    ap.add_argument("--hbm-rows", type=int, default=20_000_000, help="hbm_kernels: transactions of the input")
    ap.add_argument("--serving-scale", type=float, default=1.0, help="serving: dataset row scale")
    ap.add_argument("--serving-requests", type=int, default=256)
    ap.add_argument("--method", default=None, choices=["popcount", "tensor"])
    ap.add_argument("--tc-elem", type=int, default=None, choices=[1, 2, 4, 17, 18, 20],
                    help="tensor operands: 1 = e4m3, 2 = f16, 4 = packed e2m1 (kind::mxf4); + 16 is ignored "
                         "(default: the engine's)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparator")
    ap.add_argument("--proj-gb", type=float, default=16.0, help="device GB of projected words per chunk")
    ap.add_argument("--chunk-cands", type=int, default=None, help="candidates per chunk (default: the engine's)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU route runs")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds the CPU baseline mine may run")
    ap.add_argument("--ref-budget", type=float, default=None,
                    help="reference arm: seconds each step's mine may run (default: 180 / steps, within 20..90)")
    ap.add_argument("--no-side", action="store_true", help="skip the plain small and deep sparse side workloads")
    ap.add_argument("--no-serial", action="store_true", help="skip the one-stream mine that gives per-kernel times")
    ap.add_argument("--no-hbm", action="store_true", help="skip the AND+popcount / bitvector kernel rooflines")
    ap.add_argument("--hbm-rows-default", type=int, default=8_000_000,
                    help="transactions of the kernel-roofline input in the default line")
    ap.add_argument("--proj-cols", action="store_true",
                    help="project with the column form (etm_project: member segments by bulk copies) instead of the "
                         "row-major form")
    ap.add_argument("--no-pipeline", action="store_true",
                    help="project and count chunks in turn on one stream (per-kernel times without overlap)")
    args = ap.parse_args()
    if args.workload == "hbm_kernels":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the kernel roofline workload has no CPU arm"}))
            return
        if int(os.environ.get("RANK", "0")) == 0:
            run_hbm_kernels(args)
        return
    if args.workload == "serving":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the serving workload has no CPU arm"}))
            return
        if int(os.environ.get("RANK", "0")) == 0:
            run_serving(args)
        return
    if args.workload in TX_WORKLOADS:
        if int(os.environ.get("RANK", "0")) == 0:
            run_transactions(args)
        return
    spec = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, spec)
        return

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    pkg = _pkg()
    pkg.build_library()
    lib = pkg.load_library()
    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    method = args.method or engm.DEFAULT_METHOD
    if args.tc_elem is None:
        args.tc_elem = engm.DEFAULT_TC_ELEM
    bv = dense_k2_device(pkg, lib, spec)
    n_rows = spec["n_rows"]
    extra = {"chunk_cands": args.chunk_cands} if args.chunk_cands else {}
    eng = engm.Engine(form="batched", method=method, tc_elem=args.tc_elem, proj_bytes=int(args.proj_gb * (1 << 30)),
                      pipeline=not args.no_pipeline, proj_rows=not args.proj_cols, **extra)
    eng.profile_kernels = True

    def one(e):
        return e.mine(bv, n_rows, spec["min_support"], spec["max_length"])

    for _ in range(args.warmup):
        out = one(eng)
    torch.cuda.synchronize()
    ref_sizes = [s.n_frequent for s in out.stats]

    def barrier():
        if dist is not None:
            dist.barrier()

    eng.reset_kernel_times()
    launches0 = eng.launches
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(args.steps):
        out = one(eng)
        sizes_now = [s.n_frequent for s in out.stats]
        assert sizes_now == ref_sizes, f"level sizes changed between mines: {sizes_now} vs {ref_sizes}"
    end.record()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = start.elapsed_time(end) / args.steps
    launches = (eng.launches - launches0) // args.steps
    ms = max_over_ranks(ms, dist, "cuda")
    kern = eng.kernel_report()

    # End to end through the public API: pinned host bitvectors in, itemsets out (the engine as a user has it:
    # no per-launch timing events), right after the timed mines and before the other engines of this run exist.
    eng.profile_kernels = False
    host = torch.empty(bv.shape, dtype=torch.int64, pin_memory=True)
    host.copy_(bv.view(torch.int64))
    col_to_item = {c: c for c in range(spec["n_items"])}
    dev = torch.empty_like(bv.view(torch.int64))
    e2e_ms = []
    e2e_mine_ms = []  # the engine's own time of each call's mine (its level timers), for where a slow call went
    d2h = 0
    # Two untimed calls first: each pins one of the two result buffers that alternate while the previous result
    # is still held (a one-time cost of the process).
    for i in range(args.steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev.copy_(host, non_blocking=True)
        df = pkg.apriori(bitvecs=(dev.view(torch.uint64), col_to_item, n_rows), min_support=spec["min_support"],
                         max_length=spec["max_length"], engine=eng, warn_complexity=False)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) * 1e3
        if i > 1:
            e2e_ms.append(dt)
            e2e_mine_ms.append(sum(float(st.ms) for st in (getattr(eng, "last_stats", None) or [])))
        n_items_out = len(df)
    # Plain form (one counting launch per prefix group): the comparator.
    plain = None
    if not args.no_plain:
        pe = engm.Engine(form="plain", method=method, tc_elem=args.tc_elem, proj_bytes=int(args.proj_gb * (1 << 30)),
                         proj_rows=not args.proj_cols, **extra)
        one(pe)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        po = one(pe)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
        assert [s.n_frequent for s in po.stats] == ref_sizes
        plain = {"value": plain_s, "unit": "s", "speedup_batched": plain_s / (ms / 1e3)}
        del pe, po

    # Serial kernel times: one mine on one stream (the projection not overlapped with the Gram), so every
    # kernel's CUDA-event time is its own and the per-kernel rates are not mixed across streams.
    serial = None
    if not args.no_serial:
        se = engm.Engine(form="batched", method=method, tc_elem=args.tc_elem, proj_bytes=int(args.proj_gb * (1 << 30)),
                         pipeline=False, proj_rows=not args.proj_cols, **extra)
        se.profile_kernels = True
        one(se)
        se.reset_kernel_times()
        torch.cuda.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        so = one(se)
        s1.record()
        torch.cuda.synchronize()
        assert [s.n_frequent for s in so.stats] == ref_sizes
        sk = se.kernel_report()
        serial = {"ms_per_step": s0.elapsed_time(s1), "launches": sum(r["launches"] for r in sk.values()),
                  "kernels": {n: {"launches": r["launches"], "ms": round(r["ms"], 2), "gbs": round(r["gbs"], 1),
                                  "tflops": round(r["tflops"], 1) if r["flops"] else None}
                              for n, r in sorted(sk.items(), key=lambda kv: -kv[1]["ms"])}}
        del se, so

    # The result comes back as item ids (int64 per item), offsets (int64) and supports (float64) per itemset.
    n_sets = len(out.level1_cols) + sum(lv.n for lv in out.levels if lv.n)
    n_vals = len(out.level1_cols) + sum(lv.n * lv.k for lv in out.levels if lv.n)
    d2h = (8 * n_vals + 16 * n_sets + 8) if any(lv.n for lv in out.levels) else 0
    h2d = int(host.numel() * 8)

    peaks = _peaks()
    roof = None
    if kern:
        top = max(kern.values(), key=lambda r: r["ms"])
        per_launch_s = top["ms"] / top["launches"] / 1e3
        if top["name"] == "gram_tc":
            # Useful work: 2 x C(m,2) x rows per group, against the measured dense rate of the Gram's own MMA
            # shape and operand format (etm_tc_mma_rate: back-to-back MMAs on every SM, CUDA events).
            import ctypes

            rate = ctypes.c_double(0.0)
            st = lib.etm_tc_mma_rate(eng.tc_elem, 20000, ctypes.byref(rate), torch.cuda.current_stream().cuda_stream)
            if st != 0:
                raise RuntimeError(lib.etm_last_error().decode())
            peak = rate.value
            achieved = top["flops"] / top["launches"] / per_launch_s / 1e12
            roof = {"bound": "tensor", "kernel": top["name"], "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak,
                    "peak_source": f"measured: etm_tc_mma_rate({eng.tc_elem}) = {OPERANDS[eng.tc_elem & 7]} MMAs of "
                                   "the Gram's shape back to back on every SM (bf16 cuBLAS burst in "
                                   f"MEASURED_PEAKS.json: {peaks['bf16_tflops']:.0f})",
                    "work": "2 * C(m,2) * rows per prefix group (upper-triangle pair counts)"}
        else:
            achieved = top["bytes"] / top["launches"] / per_launch_s / 1e9
            roof = {"bound": "hbm", "kernel": top["name"], "achieved": achieved, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"]}
        ratio = DRAM_PER_ALGORITHMIC_BYTE.get(top["name"])
        traffic = ratio * top["bytes"] / top["launches"] if ratio is not None else None
        roof.update({"traffic": traffic, "traffic_unit": "bytes per launch",
                     "traffic_source": "ncu DRAM bytes per algorithmic byte on the 1M x 2048 workload, scaled"
                                       " by this run's algorithmic bytes per launch" if traffic else None,
                     "algorithmic_bytes_per_launch": top["bytes"] / top["launches"],
                     "launches_per_step": top["launches"] / args.steps,
                     "ms_per_step": top["ms"] / args.steps, "share_of_step": (top["ms"] / args.steps) / ms})

    # Parity of the benchmarked result: sampled recounts in plain PyTorch and the lattice properties.
    verm = import_module(pkg.__name__ + ".verify")
    t_v = time.perf_counter()
    rep = verm.check_mine(out, bv, n_rows, max_length=spec["max_length"], sample=10_000, seed=rank)
    exact = {"sampled": rep["sampled"], "mismatches": rep["mismatches"],
             "count_mismatches": rep["count_mismatches"], "closure_violations": rep["closure_violations"],
             "extensions_checked": rep["extensions_checked"], "extensions_frequent": rep["extensions_frequent"],
             "extension_mismatches": rep["extension_mismatches"], "level1_complete": rep["level1_complete"],
             "levels": rep["levels"], "check_s": round(time.perf_counter() - t_v, 2),
             "how": "plain-PyTorch AND + SWAR popcount recounts of up to 10,000 emitted itemsets per level; every "
                    "(k-1)-subset of each emitted; each extended by a random larger frequent item: emitted "
                    "exactly when its recount reaches min_count; level 1 complete"}

    cpu = None
    level_cands = [s.n_candidates for s in out.stats]
    recorded = LEVEL_CANDIDATES.get(args.workload)
    if recorded is not None:
        assert level_cands == recorded, (level_cands, recorded)
    side = []
    if rank == 0 and world == 1 and not args.no_cpu:
        workers = max(1, os.cpu_count() or 1)
        csr, build_s = dense_k2_host_csr(pkg, spec, workers)
        run = cpu_route_timed(csr, n_rows, spec["min_support"], spec["max_length"], args.cpu_budget, workers)
        cpu = _baseline_entry(run, workers, ROUTE_SAMPLE + f", {args.cpu_budget:.0f} s budget")
        cpu["input_build_s"] = build_s
        del csr, run
    if rank == 0 and world == 1 and not args.no_side:
        side.append(transactions_line(pkg, "plain_small_tx", max(3, args.steps), 3, with_cpu=not args.no_cpu))
        side.append(deep_sparse_line(pkg, lib, max(2, args.steps), 2, with_cpu=not args.no_cpu))
    # The AND+popcount and bitvector kernels against the HBM copy peak (the tile kernel against the popcount
    # pipe), on the deep sparse workload's shape with fewer rows.
    rooflines = None
    if rank == 0 and not args.no_hbm:
        out.levels.clear()
        torch.cuda.empty_cache()
        rooflines = {"rows": args.hbm_rows_default, "items": 2_000,
                     "kernels": hbm_kernel_rooflines(pkg, lib, n_rows=args.hbm_rows_default)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (hash-defined Bernoulli bits, on device)",
            "config": {"workload": args.workload, **spec, "method": method, "form": "batched",
                       "tc_operands": (f"{OPERANDS[args.tc_elem & 7]}, {engm.tc_block(args.tc_elem)} x "
                                       f"{engm.tc_block(args.tc_elem)} block pairs")
                       if method == "tensor" else None,
                       "l2": "inputs (1.02 GB of bitvectors) larger than L2; no flush",
                       "parallelism": "replicas" if world > 1 else "1 GPU"},
            "levels": [{"k": s.k, "candidates": s.n_candidates, "frequent": s.n_frequent, "ms": round(s.ms, 2)}
                       for s in out.stats],
            "exact": exact,
            "plain": plain,
            "e2e": {"value": statistics.median(e2e_ms) / 1e3, "unit": "s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "itemsets": n_items_out,
                    "steps_ms": [round(x, 1) for x in e2e_ms], "mine_ms": [round(x, 1) for x in e2e_mine_ms]},
            "roofline": roof,
            "rooflines": rooflines,
            "serial": serial,
            "kernels": kern,
            "cpu_baseline": cpu,
            "workloads": side,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
