"""Continuous-batching request loop: many mining requests over datasets resident on one GB300.

Each dataset's column bitvectors are built once on the device and stay
resident. Requests (dataset, min_support, max_length) arrive at any time; a
request is admitted as soon as a worker slot is free AND its estimated device
footprint fits the memory still unreserved, so work from several requests is
on the GPU at once: every slot mines on its own CUDA stream with its own
``Engine`` (its own scratch), and the kernels of different requests overlap
on the SMs. A finished request frees its slot and memory, and the queue head
is admitted immediately (continuous batching, not a queue drained one by one).

Requests on the same dataset share launches: when a slot takes the queue
head, it also takes the queued requests on that dataset whose thresholds are
within ``merge_ratio`` of the head's (and that fit the memory budget), mines
once at the lowest min_count and the longest max_length, and hands each
request the itemsets that reach its own min_count and length. That is exact:
the frequent itemsets at a threshold are those of a lower threshold whose
count reaches it (the free-set prune and generator pruning are not served
here, so no other rule applies).

Memory: admission uses an estimate of each request's device footprint; each
mine also runs under the engine's memory guard at the server's budget, so a
request whose real allocations outgrow the budget fails with MemoryError
instead of starving the others.

Latency of a request = completion time - arrival time (queueing included);
``Server.stats()`` reports p50/p99, the span from the first arrival to the
last completion and the throughput over it.

There is no counterpart in the reference (ET-Miner mines one call at a time).
"""

from __future__ import annotations

import math
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from .engine import CHUNK_CANDS, Engine, MineOutput, mining_min_count


@dataclass
class Dataset:
    """A resident dataset: device bitvectors [n_cols, ceil(N/64)], the item of each column, N."""

    bitvecs: torch.Tensor
    items: np.ndarray
    n_rows: int
    col_counts: np.ndarray | None = None

    @property
    def n_cols(self) -> int:
        return int(self.bitvecs.shape[0])

    @property
    def n_words(self) -> int:
        return int(self.bitvecs.shape[1])


@dataclass
class Job:
    rid: int
    dataset: int
    min_support: float
    max_length: int | None
    arrival: float
    footprint: int = 0
    future: Future = field(default_factory=Future)
    started: float = 0.0
    finished: float = 0.0


@dataclass
class Result:
    rid: int
    dataset: int
    levels: list[tuple[np.ndarray, np.ndarray]]
    n_rows: int
    latency_s: float
    queued_s: float
    run_s: float
    arrival: float = 0.0
    finished: float = 0.0
    batch: int = 1  # requests served by the same mine


def dataset_from_transactions(indptr: np.ndarray, items: np.ndarray, device=None) -> Dataset:
    """Build a resident dataset on the device from a transaction CSR: the item columns (deduplicated per
    row, in ascending id order) and their bitvectors (etm_build_bitvecs), all on the device."""
    import torch

    from .api import _bitvecs_of_device_csr, _frequent_csr_device

    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    n_rows = len(indptr) - 1
    row_ptr, cols, col_items, _, counts = _frequent_csr_device(np.asarray(indptr, np.int64), np.asarray(items), n_rows,
                                                               1, dev)
    with torch.cuda.device(dev):
        bv = _bitvecs_of_device_csr(row_ptr, cols, len(col_items), n_rows)
    return Dataset(bv, col_items.astype(np.int64), n_rows, counts.astype(np.int64))


class Server:
    """Admit, run and complete mining requests concurrently over resident datasets.

    ``hbm_budget`` bounds the sum of the admitted requests' estimated device
    footprints (bytes); ``slots`` bounds how many run at once. Engines keep
    their scratch between requests, so a slot's footprint estimate includes
    it.
    """

    def __init__(self, datasets: list[Dataset], *, slots: int = 4, hbm_budget: int | None = None,
                 engine_kw: dict | None = None, merge_ratio: float = 2.0, max_batch: int = 16):
        self.datasets = datasets
        self.slots = max(1, int(slots))
        #: Queued requests on the head's dataset join its mine when min_count(head) / min_count(them) is at most
        #: this (1 disables merging); at most max_batch requests per mine.
        self.merge_ratio = float(merge_ratio)
        self.max_batch = max(1, int(max_batch))
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(free * 0.8)
        self.hbm_budget = int(hbm_budget)
        kw = {"chunk_cands": 1 << 24, "proj_bytes": 1 << 30}
        kw.update(engine_kw or {})
        self.engine_kw = kw
        self._queue: deque[Job] = deque()
        self._reserved = 0
        self._running = 0
        self._lock = threading.Condition()
        self._results: list[Result] = []
        self._stop = False
        self._next_id = 0
        self._t0 = time.perf_counter()
        self._workers = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(self.slots)]
        for w in self._workers:
            w.start()

    # -- admission -------------------------------------------------------------
    def footprint(self, dataset: int, min_support: float) -> int:
        """Device bytes a request may hold at once: the padded generator copy, a chunk's
        count/class scratch, the projection scratch, and its levels (bounded by the pairs)."""
        ds = self.datasets[dataset]
        mc = mining_min_count(min_support, ds.n_rows)
        n_f = int((ds.col_counts >= mc).sum()) if ds.col_counts is not None else ds.n_cols
        ldp = max(32, (ds.n_words + 31) // 32 * 32)
        pairs = n_f * (n_f - 1) // 2
        chunk = min(self.engine_kw["chunk_cands"], max(1, pairs))
        levels = min(pairs, 1 << 26) * 12
        return int(n_f * ldp * 8 + chunk * 5 + min(self.engine_kw["proj_bytes"], n_f * ldp * 8) + levels + (64 << 20))

    def submit(self, dataset: int, min_support: float, max_length: int | None = None,
               arrival: float | None = None) -> Future:
        job = Job(self._next_id, int(dataset), float(min_support), max_length,
                  time.perf_counter() if arrival is None else arrival)
        self._next_id += 1
        job.footprint = self.footprint(job.dataset, job.min_support)
        if job.footprint > self.hbm_budget:
            job.future.set_exception(MemoryError(
                f"request {job.rid} needs ~{job.footprint / 2**30:.1f} GB, above the server's budget "
                f"of {self.hbm_budget / 2**30:.1f} GB"))
            return job.future
        with self._lock:
            self._queue.append(job)
            self._lock.notify_all()
        return job.future

    def _min_count(self, job: Job) -> int:
        return mining_min_count(job.min_support, self.datasets[job.dataset].n_rows)

    def _take(self) -> list[Job] | None:
        """The queue head and the queued requests that can share its mine (same dataset, thresholds within
        merge_ratio), once the batch's footprint fits the unreserved budget."""
        with self._lock:
            while True:
                if self._stop and not self._queue:
                    return None
                if self._queue:
                    head = self._queue[0]
                    mc0 = self._min_count(head)
                    batch = [head]
                    for job in list(self._queue)[1:]:
                        if len(batch) >= self.max_batch or self.merge_ratio <= 1.0:
                            break
                        if job.dataset == head.dataset and max(mc0, self._min_count(job)) <= self.merge_ratio * min(
                                mc0, self._min_count(job)):
                            batch.append(job)
                    # The mine runs at the batch's lowest threshold: its footprint is that request's.
                    need = max(j.footprint for j in batch)
                    if need + self._reserved <= self.hbm_budget:
                        for j in batch:
                            self._queue.remove(j)
                        batch[0].footprint, rest = need, batch[1:]
                        for j in rest:
                            j.footprint = 0
                        self._reserved += need
                        self._running += 1
                        return batch
                self._lock.wait(0.05)

    def _release(self, batch: list[Job]) -> None:
        with self._lock:
            self._reserved -= sum(j.footprint for j in batch)
            self._running -= 1
            self._lock.notify_all()

    # -- workers ---------------------------------------------------------------
    def _worker(self, slot: int) -> None:
        stream = torch.cuda.Stream()
        engine = None
        while True:
            batch = self._take()
            if batch is None:
                return
            try:
                with torch.cuda.stream(stream):
                    if engine is None:
                        engine = Engine(**self.engine_kw)
                    started = time.perf_counter()
                    ds = self.datasets[batch[0].dataset]
                    low = min(batch, key=self._min_count)
                    lengths = [j.max_length for j in batch]
                    max_len = None if any(m is None for m in lengths) else max(lengths)
                    out = engine.mine(ds.bitvecs, ds.n_rows, low.min_support, max_len,
                                      max_vram_gb=self.hbm_budget / (1 << 30))
                    levels = [(ds.items[cols], counts) for cols, counts in out.host_levels()]
                    stream.synchronize()
                finished = time.perf_counter()
                for job in batch:
                    mc = self._min_count(job)
                    mine = [(sets[keep], counts[keep]) for sets, counts in levels
                            if job.max_length is None or sets.shape[1] <= job.max_length
                            for keep in [counts >= mc] if keep.any()]
                    job.started, job.finished = started, finished
                    res = Result(job.rid, job.dataset, mine, ds.n_rows, finished - job.arrival,
                                 started - job.arrival, finished - started, job.arrival, finished, len(batch))
                    with self._lock:
                        self._results.append(res)
                    job.future.set_result(res)
            except BaseException as exc:  # the requests fail; the server keeps serving
                for job in batch:
                    if not job.future.done():
                        job.future.set_exception(exc)
            finally:
                self._release(batch)

    # -- lifecycle -------------------------------------------------------------
    def close(self, wait: bool = True) -> None:
        with self._lock:
            self._stop = True
            self._lock.notify_all()
        if wait:
            for w in self._workers:
                w.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def stats(self) -> dict:
        """p50 / p99 latency (s), throughput (requests/s over the span of the finished requests)."""
        with self._lock:
            res = list(self._results)
        if not res:
            return {"requests": 0}
        lat = np.array([r.latency_s for r in res])
        span = max(r.finished for r in res) - min(r.arrival for r in res)
        return {
            "requests": len(res),
            "throughput_rps": len(res) / span if span > 0 else math.nan,
            "mines": int(sum(1.0 / r.batch for r in res) + 0.5),
            "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()),
            "max_s": float(lat.max()),
            "queued_p99_s": float(np.percentile([r.queued_s for r in res], 99)),
            "run_p50_s": float(np.percentile([r.run_s for r in res], 50)),
            "span_s": float(span),
        }


def replay(server: Server, requests, speed: float = 1.0) -> list[Future]:
    """Submit ``requests`` (synthetic.Request) at their arrival times (scaled by 1/speed); returns futures."""
    t0 = time.perf_counter()
    futs = []
    for r in requests:
        due = t0 + r.arrival_s / speed
        delay = due - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        futs.append(server.submit(r.dataset, r.min_support, r.max_length, arrival=due))
    return futs


def percentile(values, q: float) -> float:
    return float(np.percentile(np.asarray(values, dtype=np.float64), q)) if len(values) else math.nan


__all__ = ["Dataset", "Server", "Result", "dataset_from_transactions", "replay", "CHUNK_CANDS", "MineOutput"]
