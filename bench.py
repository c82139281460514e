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
  plain         the one-launch-per-prefix-group form on the same input
  e2e           seconds per mine through apriori(bitvecs=...) with the
                bitvectors copied from pinned host memory and the itemsets
                copied back inside the timed region
  roofline      the dominant counting kernel: algorithmic bytes per launch over
                its CUDA-event time, against the measured HBM copy peak
  cpu_baseline  the CPU oracle on a bounded sample, extrapolated per row
``--impl reference`` times the CPU restatement of the reference's counting
path (the oracle) on the host cores instead, on the same workload.

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
#: capture of every launch of the 1M x 2048 dense K=2 workload (ncu --metrics dram__bytes_read.sum,
#: dram__bytes_write.sum,gpu__time_duration.sum --clock-control none -k "regex:gram_wide_kernel|project_seg_kernel"
#: python bench.py --workload dense_k2_mid --steps 1 --warmup 1 --no-plain --no-cpu --proj-gb 1
#: --chunk-cands 134217728: per mine
#: 16.21 GB against 12.66 GB for the Gram, 19.63 GB against 170.35 GB for the projection); the roofline's
#: ``traffic`` scales it to the bench's own launches by their algorithmic bytes.
DRAM_PER_ALGORITHMIC_BYTE = {"gram_tc": 16.21 / 12.66, "project": 19.63 / 170.35}


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


_MP_BV = None


def _mp_init(bv) -> None:
    global _MP_BV
    _MP_BV = bv


def _mp_count(sets) -> int:
    from oracle import miner

    miner.count_itemsets(sets, _MP_BV)
    return len(sets)


def cpu_estimate(spec, level_cands, budget_s: float = 12.0, bv_host=None, workers: int = 1) -> dict:
    """Seconds the CPU oracle's counting would take on the whole workload, from a timed sample.

    The oracle counts a candidate by ANDing its k column bitvectors and
    popcounting (count_per_candidate, core/cpu_miner.py:794-809), a cost
    that depends on k and the words per column, not on the bits. Per level
    a sample of candidates over full-length columns (the workload's own when
    ``bv_host`` is given, else random words of the same length) is timed and
    scaled by the level's candidate count; K=1 is one popcount per column.
    With ``workers`` > 1 the sample is split over that many spawned processes
    and the wall time of the whole sample is what is scaled.
    """
    from oracle import miner

    n_words = (spec["n_rows"] + 63) // 64
    rng = np.random.default_rng(1)
    if bv_host is None:
        n_s = 128
        bv = rng.integers(0, 2**63, size=(n_s, n_words), dtype=np.int64).view(np.uint64)
    else:
        n_s = min(128, bv_host.shape[0])
        bv = np.ascontiguousarray(bv_host[:n_s])
    pool = None
    if workers > 1:
        import multiprocessing as mp

        pool = mp.get_context("spawn").Pool(workers, initializer=_mp_init, initargs=(bv,))
        pool.map(_mp_count, [np.zeros((1, 2), np.int32)] * workers, chunksize=1)  # workers up and importing done

    def timed(sets: np.ndarray) -> float:
        if pool is None:
            t0 = time.perf_counter()
            miner.count_itemsets(sets, bv)
            return time.perf_counter() - t0
        parts = np.array_split(sets, workers)
        t0 = time.perf_counter()
        pool.map(_mp_count, parts, chunksize=1)
        return time.perf_counter() - t0

    per_level = []
    total = 0.0
    t_k1 = time.perf_counter()
    miner.popcount_rows(bv)
    t_k1 = (time.perf_counter() - t_k1) / n_s
    total += t_k1 * level_cands[0]
    per_level.append({"k": 1, "candidates": level_cands[0], "s_per_candidate": t_k1})
    cap = 65536 * max(1, workers)
    try:
        for k, n_c in enumerate(level_cands[1:], start=2):
            sample = 256
            while True:
                sets = np.sort(np.stack([rng.choice(n_s, size=k, replace=False) for _ in range(sample)]), axis=1)
                dt = timed(sets.astype(np.int32))
                if dt > budget_s / (2 * len(level_cands)) or sample >= cap:
                    break
                sample *= 4
            per = dt / sample
            total += per * n_c
            per_level.append({"k": k, "candidates": n_c, "s_per_candidate": per, "sampled": sample})
    finally:
        if pool is not None:
            pool.close()
            pool.join()
    return {"value": total, "unit": "s", "cores": max(1, workers), "kind": "port",
            "sample": "oracle/miner.py count_itemsets (AND + popcount per candidate, core/cpu_miner.py:794-809) "
                      f"timed on sampled candidates over {n_words:,}-word columns"
                      + (f", split over {workers} processes," if workers > 1 else ",")
                      + " scaled by each level's candidate count",
            "levels": per_level}


def max_over_ranks(value: float, dist=None, device: str = "cuda") -> float:
    """The largest of every rank's ``value`` (the replicas' slowest mine); ``value`` itself without a process
    group."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, spec) -> None:
    cands = LEVEL_CANDIDATES.get(args.workload)
    if cands is None:
        print(json.dumps({"impl": "reference", "unavailable": f"no recorded candidate counts for {args.workload}"}))
        return
    base = cpu_estimate(spec, cands, budget_s=max(6.0, 30.0 / max(1, args.steps + args.warmup)),
                        workers=max(1, os.cpu_count() or 1))
    line = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": base["value"] * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": args.workload, **spec},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


TX_METRIC = "apriori(transactions) seconds, plain small (60K x 1,000, s=0.01), exact counts"
#: Workloads mined through the transactions route (host CSR in, result frame out).
TX_WORKLOADS = {
    "plain_small_tx": dict(gen="plain_small", n_rows=60_000, n_items=1_000, min_support=0.01, max_length=None, seed=0),
}


def run_transactions(args) -> None:
    """The transactions route on the plain small workload (60K rows x 1,000 Zipf(1.1) items, s=0.01):
    seconds per ``apriori(transactions, use_gpu=True)`` call (transaction CSR on the host in, result frame
    out), the kernels it ran, exactness against the CPU oracle, and the oracle's whole mine of the same
    input timed beside it (this workload is small enough for the oracle to run in full)."""
    import torch

    from oracle import miner

    spec = TX_WORKLOADS[args.workload]
    pkg = _pkg()
    syn = pkg.synthetic
    t = getattr(syn, spec["gen"])(seed=spec["seed"])
    n_rows = t.n_rows

    def cpu_mine():
        t0 = time.perf_counter()
        res, col_items = miner.mine_transactions(t.indptr, t.items, n_rows, spec["min_support"], spec["max_length"])
        return time.perf_counter() - t0, miner.canonical(res.levels, col_items)

    if args.impl == "reference":
        cpu_s, _ = cpu_mine()
        base = {"value": cpu_s, "unit": "s", "cores": 1, "kind": "port",
                "sample": "oracle/miner.py mine_transactions: the whole mine of the workload, one core"}
        print(json.dumps({"impl": "reference", "metric": TX_METRIC, "value": cpu_s, "unit": "s", "n_gpus": args.gpus,
                          "steps": 1, "warmup": 0, "ms_per_step": cpu_s * 1e3, "higher_is_better": False,
                          "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
                          "config": {"workload": args.workload, **spec}, "cpu_baseline": base,
                          "e2e": {"value": cpu_s, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return
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

    for _ in range(max(1, args.warmup)):
        df = call()
    torch.cuda.synchronize()
    eng.reset_kernel_times()
    launches0 = eng.launches
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        df = call()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    kern = eng.kernel_report()
    cpu_s, want = cpu_mine()
    got = pkg.result_pairs(df, n_rows)
    n_sets = len(got)
    n_vals = sum(len(s) for s, _ in got)
    line = {
        "metric": TX_METRIC, "value": dt, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded plain_small generator, host CSR)",
        "config": {"workload": args.workload, **spec, "route": "transactions"},
        "levels": list(levels), "exact": got == want, "itemsets": n_sets,
        "e2e": {"value": dt, "unit": "s", "h2d_bytes_per_step": int(t.indptr.nbytes + t.items.nbytes),
                "d2h_bytes_per_step": 8 * n_vals + 16 * n_sets + 8},
        "kernels": kern, "gpu_launches": (eng.launches - launches0) // args.steps,
        "cpu_baseline": {"value": cpu_s, "unit": "s", "cores": 1, "kind": "port",
                         "sample": "oracle/miner.py mine_transactions: the whole mine of the workload, one core"},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


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
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="dense_k2", choices=sorted(WORKLOADS) + sorted(TX_WORKLOADS) + ["serving"])
    ap.add_argument("--slots", type=int, default=4, help="serving: requests on the GPU at once")
    ap.add_argument("--serving-scale", type=float, default=1.0, help="serving: dataset row scale")
    ap.add_argument("--serving-requests", type=int, default=256)
    ap.add_argument("--method", default=None, choices=["popcount", "tensor"])
    ap.add_argument("--tc-elem", type=int, default=None, choices=[1, 2, 4, 17, 18, 20],
                    help="tensor operands: 1 = e4m3, 2 = f16, 4 = packed e2m1 (kind::mxf4); + 16 is ignored "
                         "(default: the engine's)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparator")
    ap.add_argument("--proj-gb", type=float, default=8.0, help="device GB of projected words per chunk")
    ap.add_argument("--chunk-cands", type=int, default=None, help="candidates per chunk (default: the engine's)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-pipeline", action="store_true",
                    help="project and count chunks in turn on one stream (per-kernel times without overlap)")
    args = ap.parse_args()
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
                      pipeline=not args.no_pipeline, **extra)
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
        assert [s.n_frequent for s in out.stats] == ref_sizes
    end.record()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = start.elapsed_time(end) / args.steps
    launches = (eng.launches - launches0) // args.steps
    ms = max_over_ranks(ms, dist, "cuda")
    kern = eng.kernel_report()

    # Plain form (one counting launch per prefix group): the comparator.
    plain = None
    if not args.no_plain:
        pe = engm.Engine(form="plain", method=method, tc_elem=args.tc_elem, proj_bytes=int(args.proj_gb * (1 << 30)),
                         **extra)
        one(pe)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        po = one(pe)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
        assert [s.n_frequent for s in po.stats] == ref_sizes
        plain = {"value": plain_s, "unit": "s", "speedup_batched": plain_s / (ms / 1e3)}

    # End to end through the public API: pinned host bitvectors in, itemsets out.
    host = torch.empty(bv.shape, dtype=torch.int64, pin_memory=True)
    host.copy_(bv.view(torch.int64))
    col_to_item = {c: c for c in range(spec["n_items"])}
    dev = torch.empty_like(bv.view(torch.int64))
    e2e_ms = []
    d2h = 0
    for i in range(args.steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev.copy_(host, non_blocking=True)
        df = pkg.apriori(bitvecs=(dev.view(torch.uint64), col_to_item, n_rows), min_support=spec["min_support"],
                         max_length=spec["max_length"], engine=eng, warn_complexity=False)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) * 1e3
        if i > 0:
            e2e_ms.append(dt)
        n_items_out = len(df)
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
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_estimate(spec, level_cands, bv_host=bv[:128].view(torch.int64).cpu().numpy().view(np.uint64),
                           workers=max(1, os.cpu_count() or 1))

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
                    "d2h_bytes_per_step": d2h, "itemsets": n_items_out},
            "roofline": roof,
            "kernels": kern,
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
