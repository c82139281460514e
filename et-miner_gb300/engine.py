"""The level driver: ET-Miner's GPU mining loop on one GB300, over the C-ABI library.

Restates the behaviour of ``_apriori_row_split_multi_gpu``
(gpu/row_split.py:229-1185) for one device: K=1 popcounts and the free
items, then level by level the prefix groups of the generating level, the
subset test / count inference, the counting kernels, the survivor
compaction and the free-set test. Every step runs on the device; the host
only plans candidate chunks from the group sizes and reads the totals it
needs to size the next allocation.

Differences from the reference's internals (results are identical):

* The level's itemsets never leave the device between levels: candidates
  are decoded into the next level's rows by the compaction kernel, already in
  lexicographic order, so there is no host decode, lexsort or group build.
* Levels are held in "generator index" space: column ids 0..n_g-1 index the
  engine's padded copy of the generating columns (``fbv``); results map back
  to the caller's columns through ``gen_cols``.

Forms:
    "batched"  one launch per candidate chunk and kernel kind (default)
    "plain"    one counting launch per prefix group: the one-launch-per-group
               comparator the batched form is measured against
"""

from __future__ import annotations

import gc
import math
import threading
import time
import weakref
from dataclasses import dataclass, field
from fractions import Fraction

import numpy as np
import torch

from . import _lib
from ._lib import check, load_library
from .autotune import Autotuner

#: A prefix group with at most this many members is counted one warp per candidate.
SMALL_GROUP = 16
#: Suffixes per tile side of the tile-pair kernel.
TILE = 64
#: Candidates per chunk (int32 count + uint8 class each): bounds the level's dense scratch.
CHUNK_CANDS = 1 << 29
#: A group of more than SMALL_GROUP members is counted on its prefix's rows only when the prefix
#: holds less than this fraction of the transactions.
PROJ_DENSITY = 0.5
#: Device bytes of projected suffix words per chunk (two such sets alternate between the streams).
PROJ_BYTES = 16 << 30
#: Members per block of the tensor-core Gram kernel (e4m3 and f16 operands; packed e2m1 blocks hold 240):
#: a block pair (ua <= ub) is one work item.
TC_TILE = 256
#: Largest group (rows) the tensor-core Gram counts exactly: f32 holds every integer up to 2^24.
TC_MAX_ROWS = 1 << 24
PROJ_SEG_WORDS = 1024  # ETM_PROJ_SEG_WORDS: bitvector words per projection segment
OCC_TILE_WORDS = 32  # ETM_OCC_TILE_WORDS: bitvector words per occupancy tile
#: Row-wise K=2 crossover: rows' pair increments over pairs x words (the reference's K2_ROWS_MAX_R).
K2_ROWS_MAX_R = 3.95e-3
#: Row-wise K=3 crossover: rows' pair increments over K=3 candidates x words, with every candidate in one
#: chunk (the reference's K3_ROWS_MAX_R, gpu/row_split_chunks.py:145-159).
K3_ROWS_MAX_R = 2.5e-4
#: Counting method for tile-pairs: "popcount" or "tensor".
DEFAULT_METHOD = "tensor"


def min_count(min_support: float, n_rows: int) -> int:
    """ceil(s * N), s read as its shortest round-tripping decimal (core/result.py:57-79)."""
    return math.ceil(Fraction(str(min_support)) * n_rows)


def mining_min_count(min_support: float, n_rows: int) -> int:
    """The threshold the levels apply: ``min_count``, at least 1, as the CPU route does
    (core/cpu_miner.py:967-970); at 0 every pair would be "frequent" with count 0."""
    return max(1, min_count(min_support, n_rows))


def proj_stride(pcnt: np.ndarray, n_words: int) -> np.ndarray:
    """Words per member of a projected group: its prefix rows in whole words, plus up to four padded words
    per segment of PROJ_SEG_WORDS bitvector words (each segment's piece ends on a 4-word chunk), rounded up
    to 32 (at least 32)."""
    n_seg = max(1, -(-int(n_words) // PROJ_SEG_WORDS))
    return np.maximum(32, ((np.asarray(pcnt, np.int64) + 63) // 64 + 4 * n_seg + 31) // 32 * 32)


TC_MXF4 = 4  # ETM_TC_MXF4: packed e2m1 operands under kind::mxf4 (tc_elem code)
TC_WIDE = 16  # ETM_TC_WIDE: accepted in tc_elem and ignored (every code runs the block-pair kernel)
TC_BLOCKED = 32  # ETM_TC_BLOCKED: the Gram reads member rows in the projection's blocked layout
#: Packed e2m1 operands: the fastest exact form measured on GB300 (0.86 s per dense K=2 mine against 1.11 s
#: with e4m3 operands).
DEFAULT_TC_ELEM = TC_MXF4


def tc_block(tc_elem: int = DEFAULT_TC_ELEM) -> int:
    """Members per block of the Gram kernel for an element code: 240 for packed e2m1, else 256."""
    return 240 if (tc_elem & ~TC_WIDE) == TC_MXF4 else TC_TILE


def _tile_items(m: np.ndarray, method: int, tc_elem: int = DEFAULT_TC_ELEM) -> np.ndarray:
    """Work items of groups of m members: 64 x 64 tile-pairs (popcount) or Gram block pairs ua <= ub (tensor)."""
    if method == 1:
        t = tc_block(tc_elem)
        nb = (m + t - 1) // t
        return nb * (nb + 1) // 2
    nt = (m + TILE - 1) // TILE
    return nt * (nt + 1) // 2


def _p(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


@dataclass
class Level:
    """One level on the device: rows int32 [n, k] in generator-index space, counts int32 [n], free flags."""

    rows: torch.Tensor
    counts: torch.Tensor
    free: torch.Tensor | None = None

    @property
    def n(self) -> int:
        return int(self.rows.shape[0])

    @property
    def k(self) -> int:
        return int(self.rows.shape[1])


@dataclass
class LevelStats:
    k: int
    n_candidates: int
    n_frequent: int
    ms: float
    n_groups: int = 0
    n_chunks: int = 0
    launches: int = 0
    row_wise: bool = False  # counted from the transactions (row-wise K=2 / K=3 kernels)
    n_inferred: int = 0  # candidates whose count the subset test or the deduction bounds settled (class_stats)
    n_skipped: int = 0  # candidates the subset test or the bounds showed infrequent (class_stats)


@dataclass
class MineOutput:
    """Emitted levels (device tensors in generator-index space) and how to map them back.

    ``gen_cols[g]`` is the caller's column of generator index g. Level 1 is
    held as the caller's columns directly (``level1_cols``) because under the
    free-set prune it differs from the generators only by nothing, and in a
    complete run every frequent column is both.
    """

    n_rows: int
    min_count: int
    gen_cols: np.ndarray
    level1_cols: np.ndarray
    level1_counts: np.ndarray
    levels: list[Level] = field(default_factory=list)
    stats: list[LevelStats] = field(default_factory=list)

    def host_levels(self) -> list[tuple[np.ndarray, np.ndarray]]:
        """Every emitted level as (caller column ids int64 [n, k], counts int64 [n]) on the host."""
        out = []
        if len(self.level1_cols):
            out.append((self.level1_cols[:, None].astype(np.int64), self.level1_counts.astype(np.int64)))
        for lv in self.levels:
            if lv.n == 0:
                continue
            rows = lv.rows.cpu().numpy()
            out.append((self.gen_cols[rows].astype(np.int64), lv.counts.cpu().numpy().astype(np.int64)))
        return out

    def n_itemsets(self) -> int:
        return len(self.level1_cols) + sum(lv.n for lv in self.levels)

    def frame_arrays(self, item_of_col: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray, int]:
        """The result as flat arrays, built on the device and copied back once: (offsets int64 [n + 1],
        item ids [offsets[-1]] (int64, or uint64 when ``item_of_col`` is), support float64 [n]) for
        every emitted itemset in level order, and the bytes copied device to host.

        ``item_of_col[c]`` is the item id of the caller's column c.
        """
        wide = item_of_col.dtype == np.uint64

        def as_i64(a: np.ndarray) -> np.ndarray:
            a = np.ascontiguousarray(a)
            return a.view(np.int64) if wide else a.astype(np.int64)

        n1 = len(self.level1_cols)
        lv_on = [lv for lv in self.levels if lv.n > 0]
        if not lv_on:
            values = as_i64(item_of_col[self.level1_cols])
            offsets = np.arange(n1 + 1, dtype=np.int64)
            support = self.level1_counts.astype(np.float64) / max(1, self.n_rows)
            return offsets, values.view(np.uint64) if wide else values, support, 0
        dev = lv_on[0].rows.device
        table = torch.from_numpy(as_i64(item_of_col[self.gen_cols])).to(dev)
        vparts = [torch.from_numpy(as_i64(item_of_col[self.level1_cols])).to(dev)]
        cparts = [torch.from_numpy(self.level1_counts.astype(np.int64)).to(dev)]
        oparts = [torch.arange(0, n1 + 1, dtype=torch.int64, device=dev)]
        base = n1
        for lv in lv_on:
            vparts.append(table[lv.rows.reshape(-1).long()])
            cparts.append(lv.counts.to(torch.int64))
            oparts.append(base + lv.k * torch.arange(1, lv.n + 1, dtype=torch.int64, device=dev))
            base += lv.k * lv.n
        values_d = torch.cat(vparts)
        support_d = torch.cat(cparts).to(torch.float64) / max(1, self.n_rows)
        offsets_d = torch.cat(oparts)
        values, support, offsets = _copy_to_host(values_d, support_d, offsets_d)
        d2h = values.nbytes + support.nbytes + offsets.nbytes
        return offsets, values.view(np.uint64) if wide else values, support, d2h


#: Results at least this large come back through page-locked host memory.
PINNED_RESULT_BYTES = 64 << 20


class _PinnedPool:
    """Page-locked host buffers for results, shared by the engines of the process. A buffer is handed out again
    only once every numpy array made from it has been dropped (weak references), so a result never shares
    memory with a live earlier result, and steady-state calls pin nothing new; at most ``max_buffers`` are
    kept (past that, results come back through pageable memory)."""

    def __init__(self, max_buffers: int = 4):
        self.lock = threading.Lock()
        self.entries: list[list] = []  # [uint8 page-locked tensor, [weak references or a busy marker]]
        self.max_buffers = max_buffers

    @staticmethod
    def _free(entry) -> bool:
        return all(r() is None for r in entry[1])

    def arrays(self, tensors: list[torch.Tensor]) -> list[np.ndarray] | None:
        sizes = [t.numel() * t.element_size() for t in tensors]
        offs, total = [], 0
        for n in sizes:
            offs.append(total)
            total += -(-n // 256) * 256
        with self.lock:
            have = any(e[0].numel() >= total and self._free(e) for e in self.entries)
            busy = bool(self.entries)
        if not have and busy:
            # A dropped result held in a reference cycle is freed only by the collector: collect once (outside
            # the lock: finalizers may run) before pinning another buffer, which takes longer than a collection.
            gc.collect()
        with self.lock:
            entry = next((e for e in self.entries if e[0].numel() >= total and self._free(e)), None)
            if entry is None:
                if len(self.entries) >= self.max_buffers:
                    free = [e for e in self.entries if self._free(e)]
                    if not free:
                        return None
                    self.entries.remove(free[0])
                entry = [torch.empty(total, dtype=torch.uint8, pin_memory=True), []]
                self.entries.append(entry)
            entry[1] = [lambda: True]  # busy while the copies run
        buf = entry[0]
        views = [buf[o:o + n].view(t.dtype).view(t.shape) for o, n, t in zip(offs, sizes, tensors)]
        for v, t in zip(views, tensors):
            v.copy_(t, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        out = [v.numpy() for v in views]
        with self.lock:
            entry[1] = [weakref.ref(a) for a in out]
        return out


_PINNED = _PinnedPool()


def _copy_to_host(*tensors: torch.Tensor) -> list[np.ndarray]:
    """Device tensors as host numpy arrays: large results through the page-locked pool (full-rate copies, no
    page faults on fresh memory), small ones (or with the pool exhausted) through ``.cpu()``."""
    if sum(t.numel() * t.element_size() for t in tensors) >= PINNED_RESULT_BYTES:
        got = _PINNED.arrays(list(tensors))
        if got is not None:
            return got
    return [t.cpu().numpy() for t in tensors]


class _Scratch:
    """Reusable device buffers, grown on demand (torch allocations: plumbing only)."""

    def __init__(self, device: torch.device):
        self.device = device
        self.bufs: dict[str, torch.Tensor] = {}

    def get(self, name: str, n: int, dtype: torch.dtype) -> torch.Tensor:
        t = self.bufs.get(name)
        n = max(int(n), 1)
        if t is None or t.dtype != dtype or t.numel() < n:
            t = torch.empty(int(n * 1.25) + 16, dtype=dtype, device=self.device)
            self.bufs[name] = t
        return t[:n]


def host_rss_gb() -> float:
    """Resident set size of this process in GB (/proc/self/status; 0 where it cannot be read)."""
    try:
        with open("/proc/self/status") as f:
            for line in f:
                if line.startswith("VmRSS:"):
                    return int(line.split()[1]) / (1 << 20)
    except OSError:
        pass
    return 0.0


def check_memory_guard(k: int, ram_gb: float, vram_gb: float, max_ram_gb: float | None,
                       max_vram_gb: float | None) -> None:
    """Raise MemoryError when a level left the process over a memory limit (gpu/row_split.py:467-487): the
    lattice is incomplete at that point, so it is not returned."""
    for used, limit, what, remedy in (
        (ram_gb, max_ram_gb, "RAM", "lower max_length or mine fewer levels per call"),
        (vram_gb, max_vram_gb, "VRAM", "lower max_length, or lower the engine's chunk and projection budgets"),
    ):
        if limit is not None and used > limit:
            raise MemoryError(
                f"Memory guard tripped after K={k}: {what}={used:.1f}GB exceeds max_{what.lower()}_gb={limit}GB. "
                f"The lattice is INCOMPLETE at this point, so it is not returned. Raise max_{what.lower()}_gb, "
                f"or {remedy}.")


def scan_words(n: int) -> int:
    return (max(n, 1) + 4095) // 4096 + 2


def as_device_bitvecs(bitvecs) -> tuple[int, tuple[int, int], object]:
    """(device pointer, (n_cols, n_words), owner) of a C-contiguous uint64 device array.

    Accepts a torch CUDA tensor (uint64 or int64) or any object exposing
    ``__cuda_array_interface__`` with typestr ``<u8``.
    """
    if isinstance(bitvecs, torch.Tensor):
        if not bitvecs.is_cuda:
            raise TypeError("bitvecs must live on a CUDA device")
        if bitvecs.dtype not in (torch.uint64, torch.int64):
            raise ValueError(f"bitvecs must be uint64, got {bitvecs.dtype}")
        if bitvecs.dim() != 2 or not bitvecs.is_contiguous():
            raise ValueError("bitvecs must be a C-contiguous 2-D array")
        return bitvecs.data_ptr(), (int(bitvecs.shape[0]), int(bitvecs.shape[1])), bitvecs
    cai = getattr(bitvecs, "__cuda_array_interface__", None)
    if cai is None:
        raise TypeError(f"bitvecs must expose __cuda_array_interface__, got {type(bitvecs).__name__}")
    shape = tuple(cai["shape"])
    if len(shape) != 2:
        raise ValueError(f"bitvecs must be 2D (n_cols, n_u64s), got {len(shape)}D")
    if cai["typestr"] not in ("<u8", "|u8"):
        raise ValueError(f"bitvecs must be uint64, got {cai['typestr']}")
    strides = cai.get("strides")
    if strides is not None and tuple(strides) != (shape[1] * 8, 8):
        raise ValueError("bitvecs must be C-contiguous")
    return int(cai["data"][0]), (int(shape[0]), int(shape[1])), bitvecs


class Engine:
    """One device's mining state: the library, scratch buffers and the counting choices."""

    def __init__(self, device: torch.device | int | None = None, *, method: str = DEFAULT_METHOD,
                 form: str = "batched", chunk_cands: int = CHUNK_CANDS, small_group: int = SMALL_GROUP,
                 project: bool = True, proj_density: float = PROJ_DENSITY, proj_bytes: int = PROJ_BYTES,
                 tc_elem: int = DEFAULT_TC_ELEM, pipeline: bool = True, autotune: "Autotuner | bool | None" = None,
                 fused: bool = True, deduction_bounds: bool = True, proj_rows: bool = True):
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 engine needs a CUDA device; there is no CPU fallback")
        self.lib = load_library()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else
                                   (device.index if isinstance(device, torch.device) else int(device)))
        if method not in ("popcount", "tensor"):
            raise ValueError(f"method must be 'popcount' or 'tensor', got {method!r}")
        if form not in ("batched", "plain"):
            raise ValueError(f"form must be 'batched' or 'plain', got {form!r}")
        self.method = method
        self.form = form
        self.chunk_cands = int(chunk_cands)
        self.small_group = int(small_group)
        self.project = bool(project)
        self.proj_density = float(proj_density)
        self.proj_bytes = int(proj_bytes)
        #: Tensor-core operand element: 1 = e4m3 (kind::f8f6f4), 2 = f16 (kind::f16), 4 = packed e2m1 (kind::mxf4).
        if (int(tc_elem) & ~TC_WIDE) not in (1, 2, TC_MXF4):
            raise ValueError(f"tc_elem must be 1 (e4m3), 2 (f16) or 4 (e2m1), optionally | 16; got {tc_elem}")
        self.tc_elem = int(tc_elem)
        #: Batched form with the column projection (proj_rows=False): project chunk c+1 on a side stream while
        #: chunk c is counted.
        self.pipeline = bool(pipeline)
        #: Fused threshold: the counting kernels write only the counts reaching min_count and a survivor bit each;
        #: compaction scans the bitmask (a 32nd of the dense counts). False: dense counts, dense compaction.
        self.fused = bool(fused)
        #: Under count inference, settle candidates by the deduction bounds of depth <= 3 from levels k-2 and
        #: k-3 (on by default in the reference's GPU route, gpu/row_split.py:541-546, 629); needs fused.
        self.deduction_bounds = bool(deduction_bounds)
        #: Projection from a row-major copy of the generating columns (etm_project_rows, 32 x 32 bit transposes
        #: over the prefix rows) instead of gathering every member's segment words (etm_project); the copy is
        #: built once per mine and skipped when it would exceed ``rows_copy_max_bytes``.
        self.proj_rows = bool(proj_rows)
        #: Row order of the bitvectors that ``apriori(transactions, ...)`` builds for this engine: "keep" (input
        #: order) or "lex" (the rows sorted by their most frequent columns, with the tile-occupancy skip; the
        #: reference's choice). Counts never depend on it. Measured on the deep sparse transactions (2M rows),
        #: lex halves the per-candidate counting but gathers each prefix's rows into few projection segments,
        #: whose units then run unbalanced (projection 0.43 -> 0.96 ms): 42.3 against 43.8 ms per call, so the
        #: input order is the default.
        self.row_order = "keep"
        #: Under "lex", fewer rows than this keep their order: a few tiles per column leave the occupancy little
        #: to skip, and the keys, sorts and permutation would cost more than they save.
        self.lex_min_rows = 1 << 18
        self.rows_copy_max_bytes = 32 << 30
        self._xt = None
        self._xt_key = None
        #: (occupancy, words per column) of the mine's generating columns, when it asked for one.
        self._occ = None
        #: (level k-2, level k-3 or None, N) of the level being counted, for the deduction bounds.
        self._deep = None
        #: When set, each level's stats count the candidates classified INFER and SKIP (one extra pass per chunk).
        self.class_stats = False
        #: K=2 counts row-wise from the transactions (when given) while
        #: sum C(len,2) / (pairs x words) is below this (gpu/row_split_chunks.py:130-142); 0 disables.
        self.k2_rows_max_r = K2_ROWS_MAX_R
        self.k3_rows_max_r = K3_ROWS_MAX_R
        self._k2_rows = None
        self._rows_input = None
        #: Counting settings chosen per level shape by timing (None: the fixed defaults).
        self.autotuner = Autotuner() if autotune is True else (autotune or None)
        self.scratch = _Scratch(self.device)
        self.launches = 0
        #: When set, every counting / compaction launch is bracketed by CUDA events on its stream.
        self.profile_kernels = False
        self._events: list[tuple] = []
        self.used_tensor = False
        #: Set when a kernel with bounded device waits (the Gram, the projection) ran since the last status read.
        self._waits_pending = False
        self._side: torch.cuda.Stream | None = None

    def _sms(self) -> int:
        if getattr(self, "_sm_count", None) is None:
            self._sm_count = max(1, int(self.lib.etm_device_sm_count()))
        return self._sm_count

    def _side_stream(self) -> torch.cuda.Stream:
        """The stream projection runs on beside the counting kernels (created on first use)."""
        if self._side is None:
            self._side = torch.cuda.Stream(device=self.device)
        return self._side

    # -- kernel timing ----------------------------------------------------------
    def _launch(self, name: str, nbytes: int, fn, flops: float = 0.0):
        """Run ``fn`` (one library call), timing it with CUDA events when profiling."""
        if not self.profile_kernels:
            return fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        st = fn()
        e1.record()
        self._events.append((name, e0, e1, int(nbytes), float(flops)))
        return st

    def reset_kernel_times(self) -> None:
        self._events = []

    def kernel_report(self) -> dict:
        """Per kernel: launches, total ms (CUDA events on the launching stream), algorithmic bytes."""
        torch.cuda.synchronize()
        out: dict[str, dict] = {}
        for name, e0, e1, nbytes, flops in self._events:
            r = out.setdefault(name, {"name": name, "launches": 0, "ms": 0.0, "bytes": 0, "flops": 0.0})
            r["launches"] += 1
            r["ms"] += e0.elapsed_time(e1)
            r["bytes"] += nbytes
            r["flops"] += flops
        for r in out.values():
            r["gbs"] = r["bytes"] / (r["ms"] / 1e3) / 1e9 if r["ms"] > 0 else 0.0
            r["tflops"] = r["flops"] / (r["ms"] / 1e3) / 1e12 if r["ms"] > 0 else 0.0
        return out

    # -- K = 1 -----------------------------------------------------------------
    def column_counts(self, ptr: int, n_cols: int, n_words: int, ld: int) -> np.ndarray:
        out = self.scratch.get("colcounts", n_cols, torch.int64)
        check(self.lib.etm_popcount_cols(ptr, n_cols, n_words, ld, _p(out), _stream()), "etm_popcount_cols")
        self.launches += 1
        return out.cpu().numpy().copy()

    def gather(self, ptr: int, ld: int, cols: np.ndarray, n_words: int) -> tuple[torch.Tensor, int]:
        ldp = max(32, (n_words + 31) // 32 * 32)
        fbv = torch.empty((max(len(cols), 1), ldp), dtype=torch.int64, device=self.device)
        cols_d = torch.from_numpy(cols.astype(np.int32)).to(self.device)
        check(self.lib.etm_gather_cols(ptr, ld, _p(cols_d), len(cols), n_words, _p(fbv), ldp, _stream()),
              "etm_gather_cols")
        self.launches += 1
        return fbv, ldp

    # -- K >= 2 ----------------------------------------------------------------
    def groups(self, gen: Level):
        n, width = gen.n, gen.k
        grp_first = self.scratch.get("grp_first", n, torch.int64)
        grp_size = self.scratch.get("grp_size", n, torch.int32)
        cand_off = self.scratch.get("cand_off", n + 1, torch.int64)
        counters = self.scratch.get("counters", 2, torch.int64)
        ws = self.scratch.get("ws_groups", 3 + scan_words(n), torch.int64)
        check(self.lib.etm_level_groups(_p(gen.rows), n, width, _p(grp_first), _p(grp_size), _p(cand_off),
                                        _p(counters), _p(ws), ws.numel(), _stream()), "etm_level_groups")
        self.launches += 10
        G, total = (int(x) for x in counters.cpu().tolist())
        return G, total, grp_first, grp_size, cand_off

    def _work(self, ids: np.ndarray, weights: np.ndarray) -> tuple[torch.Tensor, torch.Tensor]:
        off = np.zeros(len(ids) + 1, dtype=np.int64)
        np.cumsum(weights, out=off[1:])
        both = torch.from_numpy(np.concatenate([ids.astype(np.int64), off])).to(self.device, non_blocking=False)
        return both[: len(ids)], both[len(ids):]

    def prefix_counts(self, fbv, ldp: int, n_words: int, gen: Level, grp_first, ids: np.ndarray) -> np.ndarray:
        """Rows holding each listed group's prefix (popcount of the AND of its prefix columns)."""
        wg = torch.from_numpy(ids.astype(np.int64)).to(self.device)
        out = self.scratch.get("prefix_counts", len(ids), torch.int64)
        st = self._launch("prefix_counts", len(ids) * (gen.k - 1) * n_words * 8, lambda: self.lib.etm_prefix_counts(
            _p(fbv), ldp, n_words, _p(gen.rows), gen.k, _p(grp_first), _p(wg), len(ids), _p(out), *self._occ_args(),
            _stream()))
        check(st, "etm_prefix_counts")
        self.launches += 1
        return out.cpu().numpy().copy()

    def tile_occupancy(self, fbv: torch.Tensor, ldp: int, n_words: int) -> tuple[torch.Tensor, int]:
        """(occ int64 [n_cols][occ_ld], occ_ld): per generating column, one bit per tile of ETM_OCC_TILE_WORDS
        words holding a row of it (etm_tile_occupancy; gpu/kernels/occupancy.py:37-58)."""
        n_g = int(fbv.shape[0])
        occ_ld = max(1, -(-(-(-n_words // OCC_TILE_WORDS)) // 64))
        occ = torch.empty((n_g, occ_ld), dtype=torch.int64, device=self.device)
        st = self._launch("tile_occupancy", n_g * (n_words + occ_ld) * 8, lambda: self.lib.etm_tile_occupancy(
            _p(fbv), n_g, n_words, ldp, _p(occ), occ_ld, _stream()))
        check(st, "etm_tile_occupancy")
        self.launches += 1
        return occ, occ_ld

    def _occ_args(self) -> tuple:
        """The (occ, occ_ld) arguments of the prefix and per-candidate kernels: the mine's tile occupancy, or none."""
        return (None, 0) if self._occ is None else (_p(self._occ[0]), self._occ[1])

    def _rows_copy(self, fbv: torch.Tensor, ldp: int, n_words: int):
        """(xt, ldr): the row-major copy of the mine's generating columns that etm_project_rows reads (word c of
        row r holds bit r of columns 32 c .. 32 c + 31), built on the current stream at its first use in a mine;
        None when it would exceed ``rows_copy_max_bytes``."""
        n_g = int(fbv.shape[0])
        key = (fbv.data_ptr(), n_words, n_g)
        if self._xt_key == key:
            return self._xt
        ldr = max(4, -(-(-(-n_g // 32)) // 4) * 4)
        nbytes = n_words * 64 * ldr * 4
        self._xt, self._xt_key = None, key
        if nbytes > self.rows_copy_max_bytes:
            return None
        xt = torch.empty((n_words * 64, ldr), dtype=torch.int32, device=self.device)
        st = self._launch("rows_transpose", n_g * n_words * 8 + nbytes, lambda: self.lib.etm_rows_transpose(
            _p(fbv), ldp, n_words, n_g, _p(xt), ldr, _stream()))
        check(st, "etm_rows_transpose")
        self.launches += 1
        self._xt = (xt, ldr)
        return self._xt

    def _prep_projected(self, fbv, ldp, n_words, gen, grp_first, grp_size, gids, sizes, pcnt, method, buf: int = 0,
                        xt=None):
        """Segment offsets and projected member words of the listed groups (two launches on the current stream).

        Returns what ``_count_prepped`` needs. ``buf`` selects one of two scratch sets, so the
        projection of the next chunk can run while the current one is counted. ``xt``: the row-major copy
        (``_rows_copy``) for the row-major projection, else the column form runs.
        """
        width = gen.k
        # Longest prefixes first: the Gram's CTAs claim block pairs in this order, so the last ones are short.
        gids = gids[np.argsort(-pcnt[gids], kind="stable")]
        m = sizes[gids]
        cnt = pcnt[gids]
        n_seg = max(1, -(-n_words // PROJ_SEG_WORDS))
        cl = proj_stride(cnt, n_words)
        # The Gram reads blocked rows (blocks of its block size, chunk by chunk); rows past m are not written.
        blk = tc_block(self.tc_elem) if method == 1 else 0
        m_rows = -(-m // blk) * blk if blk else m
        cb = np.zeros(len(gids) + 1, np.int64)
        np.cumsum(m_rows * cl, out=cb[1:])
        toff = np.zeros(len(gids) + 1, np.int64)
        np.cumsum(_tile_items(m, method, self.tc_elem), out=toff[1:])
        n = len(gids)
        # cwords starts as the bound (whole words of the prefix rows plus one padded word per segment);
        # etm_prefix_segments overwrites it with the exact padded length.
        host = np.concatenate([gids.astype(np.int64), toff, cb[:-1], (cnt + 63) // 64 + 4 * n_seg, cl])
        d = torch.from_numpy(host).to(self.device)
        wg, wo = d[:n], d[n:2 * n + 1]
        cbase, cwords, cld = d[2 * n + 1:3 * n + 1], d[3 * n + 1:4 * n + 1], d[4 * n + 1:5 * n + 1]
        seg_off = self.scratch.get(f"proj_seg_{buf}", n * (n_seg + 1), torch.int64)
        proj_counter = self.scratch.get(f"proj_counter_{buf}", 1, torch.int64)
        cbuf = self.scratch.get(f"proj_cbuf_{buf}", int(cb[-1]), torch.int64)
        st = self._launch("prefix_segments", int(n * (width - 1) * n_words * 8),
                          lambda: self.lib.etm_prefix_segments(_p(fbv), ldp, n_words, _p(gen.rows), width,
                                                               _p(grp_first), _p(wg), n, _p(seg_off), _p(cwords),
                                                               *self._occ_args(), _stream()))
        check(st, "etm_prefix_segments")
        if xt is not None:
            # Algorithmic bytes: the prefix columns' words and the prefix rows' row-major words read once, the
            # member strides written.
            xt_t, ldr = xt
            st = self._launch("project_rows", int(n * (width - 1) * n_words * 8 + (cnt * ldr).sum() * 4
                                                  + (m * cl).sum() * 8),
                              lambda: self.lib.etm_project_rows(
                                  _p(fbv), ldp, n_words, _p(xt_t), ldr, _p(gen.rows), width, _p(grp_first),
                                  _p(grp_size), _p(wg), n, _p(seg_off), _p(cbase), _p(cld), blk, _p(cbuf),
                                  _stream()))
            check(st, "etm_project_rows")
            xt_t.record_stream(torch.cuda.current_stream())
            self._waits_pending = True
            self.launches += 2
            return dict(d=d, cbuf=cbuf, cbase=cbase, cwords=cwords, cld=cld, wg=wg, wo=wo, n=n,
                        n_tiles=int(toff[-1]), blocked=bool(blk), nbytes=int((m * ((cnt + 63) // 64)).sum() * 8),
                        macs=float((m * (m - 1) / 2 * cnt.astype(np.float64)).sum()))
        # Algorithmic bytes: every member's column words and the prefix words read once, the strides written.
        st = self._launch("project", int(((m + width - 1) * n_words).sum() * 8 + (m * cl).sum() * 8),
                          lambda: self.lib.etm_project_blocked(
                              _p(fbv), ldp, n_words, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(wg), n,
                              _p(seg_off), _p(cbase), _p(cld), blk, _p(cbuf), _p(proj_counter), _stream())
                          if blk else self.lib.etm_project(
                              _p(fbv), ldp, n_words, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(wg), n,
                              _p(seg_off), _p(cbase), _p(cld), _p(cbuf), _p(proj_counter), _stream()))
        check(st, "etm_project")
        self._waits_pending = True
        self.launches += 2
        return dict(d=d, cbuf=cbuf, cbase=cbase, cwords=cwords, cld=cld, wg=wg, wo=wo, n=n, n_tiles=int(toff[-1]),
                    blocked=bool(blk),
                    nbytes=int((m * ((cnt + 63) // 64)).sum() * 8),
                    macs=float((m * (m - 1) / 2 * cnt.astype(np.float64)).sum()))

    def _count_prepped(self, prep, grp_size, cand_off, base, cls, counts, method, sel=None):
        """The tile-pair counts of a prepared projection (one launch on the current stream).

        Every tensor the projection made on the side stream and the counting reads here is recorded on this
        stream, so the caching allocator does not hand its memory to a later side-stream allocation (a grown
        scratch buffer) while this stream may still read it.
        """
        cur = torch.cuda.current_stream()
        prep["d"].record_stream(cur)
        prep["cbuf"].record_stream(cur)
        self._count_words(prep["cbuf"], prep["cbase"], prep["cwords"], prep["cld"], grp_size, cand_off, prep["wg"],
                          prep["wo"], prep["n"], prep["n_tiles"], base, cls, counts, method, prep["nbytes"],
                          prep["macs"], sel, prep["blocked"])

    def _count_projected(self, fbv, ldp, n_words, gen, grp_first, grp_size, cand_off, gids, sizes, pcnt, base, cls,
                         counts, method, sel=None, xt=None):
        """Row lists, projected suffix words and tile-pair counts of the listed groups (one launch each)."""
        prep = self._prep_projected(fbv, ldp, n_words, gen, grp_first, grp_size, gids, sizes, pcnt, method, 0, xt)
        self._count_prepped(prep, grp_size, cand_off, base, cls, counts, method, sel)

    def _count_words(self, cbuf, cbase, cwords, cld, grp_size, cand_off, wg, wo, n, n_tiles, base, cls, counts,
                     method, nbytes, macs, sel=None, blocked: bool = False):
        """Tile-pair counts over member words laid out as cbuf[cbase[wi] + i * cld[wi]]: tensor or popcount.

        ``macs`` is the useful work: one multiply-add per candidate pair and row (sum of C(m,2) x rows).
        ``sel`` = (min_count, survivor bitmask) selects the fused-threshold form; ``blocked``: the rows are in
        the projection's blocked layout (tensor method).
        """
        elem = self.tc_elem | (TC_BLOCKED if blocked else 0)
        if method == 1:
            # The work counter lets the Gram's CTAs claim block pairs dynamically (one per engine: the Gram
            # launches of an engine run in turn on its main stream).
            counter = self.scratch.get("tc_work_counter", 1, torch.int64)
            if sel is None:
                fn = lambda: self.lib.etm_count_tiles_tc(  # noqa: E731
                    _p(cbuf), _p(cbase), _p(cwords), _p(cld), _p(grp_size), _p(cand_off), _p(wg), _p(wo), n, n_tiles,
                    base, _p(cls), elem, _p(counts), _p(counter), _stream())
            else:
                fn = lambda: self.lib.etm_count_tiles_tc_sel(  # noqa: E731
                    _p(cbuf), _p(cbase), _p(cwords), _p(cld), _p(grp_size), _p(cand_off), _p(wg), _p(wo), n, n_tiles,
                    base, _p(cls), elem, sel[0], _p(counts), _p(sel[1]), _p(counter), _stream())
            check(self._launch("gram_tc", nbytes, fn, flops=2 * macs), "etm_count_tiles_tc")
            self.used_tensor = True
            self._waits_pending = True
        else:
            if sel is None:
                fn = lambda: self.lib.etm_count_tiles_proj(  # noqa: E731
                    _p(cbuf), _p(cbase), _p(cwords), _p(cld), _p(grp_size), _p(cand_off), _p(wg), _p(wo), n, base,
                    _p(cls), 0, _p(counts), _stream())
            else:
                fn = lambda: self.lib.etm_count_tiles_proj_sel(  # noqa: E731
                    _p(cbuf), _p(cbase), _p(cwords), _p(cld), _p(grp_size), _p(cand_off), _p(wg), _p(wo), n, base,
                    _p(cls), sel[0], _p(counts), _p(sel[1]), _stream())
            check(self._launch("count_tiles_proj", nbytes, fn), "etm_count_tiles_proj")
        self.launches += 1

    def count_level(self, gen: Level, fbv: torch.Tensor, ldp: int, n_words: int, mc: int,
                    infer: bool, prune: bool, n_rows: int | None = None) -> tuple[Level, LevelStats]:
        """Count every candidate of the level generated by ``gen``; returns the survivors (k = gen.k + 1).

        Groups with at most ``small_group`` members are counted one warp per
        candidate; larger groups by 64 x 64 tile-pairs, on the prefix's rows
        only (projected) when the prefix holds less than ``proj_density`` of the
        transactions, else on the full bitvectors with the prefix ANDed in.
        Chunks of whole groups bound the dense count scratch (``chunk_cands``)
        and the projection scratch (``proj_bytes``).
        """
        t0 = time.perf_counter()
        width = gen.k
        n_rows = n_words * 64 if n_rows is None else n_rows
        G, total, grp_first, grp_size, cand_off = self.groups(gen)
        stats = LevelStats(width + 1, total, 0, 0.0, G)
        if total == 0:
            stats.ms = (time.perf_counter() - t0) * 1e3
            empty = Level(torch.empty((0, width + 1), dtype=torch.int32, device=self.device),
                          torch.empty(0, dtype=torch.int32, device=self.device))
            return empty, stats
        sizes = grp_size[:G].cpu().numpy().astype(np.int64)
        offs = cand_off[: G + 1].cpu().numpy()
        args = (gen, fbv, ldp, n_words, mc, infer, prune, n_rows, G, total, grp_first, grp_size, cand_off, sizes,
                offs, stats)
        tuner = self.autotuner
        if tuner is None or total < tuner.min_candidates:
            level = self._count_groups(*args)
        else:
            key = tuner.key(width + 1, n_words, sizes, total, self.method)
            if key in tuner.cache:
                with self._settings(tuner.cache[key]):
                    level = self._count_groups(*args)
            else:
                # First level of this shape: count it under every setting, keep the fastest.
                best = None
                for setting in tuner.settings(self.method):
                    with self._settings(setting):
                        torch.cuda.synchronize()
                        t1 = time.perf_counter()
                        trial = self._count_groups(*args)
                        torch.cuda.synchronize()
                        dt = time.perf_counter() - t1
                    tuner.trials.append({"key": key, **setting, "s": dt})
                    if best is None or dt < best[0]:
                        best = (dt, setting, trial)
                tuner.cache[key] = best[1]
                level = best[2]
        stats.ms = (time.perf_counter() - t0) * 1e3
        stats.n_frequent = level.n
        return level, stats

    def _settings(self, setting: dict):
        """Context manager applying tuned attributes (small_group, proj_density) for one count."""
        engine = self

        class _Apply:
            def __enter__(self):
                self.saved = {k: getattr(engine, k) for k in setting}
                for k, v in setting.items():
                    setattr(engine, k, v)

            def __exit__(self, *exc):
                for k, v in self.saved.items():
                    setattr(engine, k, v)

        return _Apply()

    def _count_groups(self, gen, fbv, ldp, n_words, mc, infer, prune, n_rows, G, total, grp_first, grp_size,
                      cand_off, sizes, offs, stats) -> Level:
        """The counting of a level's candidates given its groups (see ``count_level``)."""
        width = gen.k
        stats.n_chunks = 0
        out_rows = torch.empty((0, width + 1), dtype=torch.int32, device=self.device)
        out_counts = torch.empty(0, dtype=torch.int32, device=self.device)
        # The subset test has prefix subsets to look up only from K=3 on.
        classify = (infer or prune) and width >= 2
        mode = (1 if prune or infer else 0) | (2 if infer else 0)
        deep = self._deep if (infer and self.deduction_bounds and self.fused and width + 1 <= 24) else None
        if deep is not None:
            mode |= 4  # ETM_SUBSET_BOUNDS
        big = sizes > self.small_group
        tensor = self.method == "tensor"
        pcnt = np.zeros(G, np.int64)
        proj = np.zeros(G, bool)
        ri = self._rows_input
        # K=3 from the transactions: each row adds 1 to the candidates it holds (sparse rows, one chunk).
        k3_rows = (width == 2 and ri is not None and self.k3_rows_max_r > 0 and total <= self.chunk_cands
                   and ri["pair_work"] < self.k3_rows_max_r * total * n_words)
        stats.row_wise = stats.row_wise or k3_rows
        if not k3_rows and (self.project or tensor) and width >= 2 and big.any():
            ids_big = np.flatnonzero(big)
            pcnt[ids_big] = self.prefix_counts(fbv, ldp, n_words, gen, grp_first, ids_big)
            if tensor:
                # The tensor cores count projected words; a prefix past 2^24 rows stays on popcount.
                proj = big & (pcnt <= TC_MAX_ROWS)
            else:
                proj = big & (pcnt < self.proj_density * n_rows)
        pwords = proj_stride(pcnt, n_words)
        blk = tc_block(self.tc_elem) if tensor else 0
        pbytes = np.where(proj, (-(-sizes // blk) * blk if blk else sizes) * pwords * 8, 0)
        pcum = np.zeros(G + 1, np.int64)
        np.cumsum(pbytes, out=pcum[1:])
        cap = int(min(total, max(1 << 16, 2 * gen.n)))
        out_rows = torch.empty((cap, width + 1), dtype=torch.int32, device=self.device)
        out_counts = torch.empty(cap, dtype=torch.int32, device=self.device)
        acc = self.scratch.get("acc", 1, torch.int64)
        acc.zero_()
        n_out = 0
        method = 1 if tensor else 0
        # K=2 on the tensor cores: the one group of every generator, its members the padded columns.
        whole_tc = tensor and width == 1 and n_rows <= TC_MAX_ROWS
        # Chunks: whole groups within both budgets (at least one group each).
        chunks = []
        g0 = 0
        while g0 < G:
            g1c = int(np.searchsorted(offs, offs[g0] + self.chunk_cands, side="right")) - 1
            g1p = int(np.searchsorted(pcum, pcum[g0] + self.proj_bytes, side="right")) - 1
            g1 = max(min(g1c, g1p), g0 + 1)
            chunks.append((g0, g1))
            g0 = g1
        # The row-major copy for the projection, made on the main stream before any side-stream work reads it.
        xt = self._rows_copy(fbv, ldp, n_words) if (self.proj_rows and proj.any()) else None
        # Batched form with the column projection: the projection of chunk c+1 runs on a side stream while chunk
        # c is counted; two scratch sets alternate. The row-major projection stays on the main stream: it is
        # short, and the Gram's CTAs leave no room on their SMs for it (measured: 0.563 s per dense K=2 mine
        # with the side stream, 0.545 s without).
        pipelined = self.pipeline and self.form == "batched" and proj.any() and xt is None
        main = torch.cuda.current_stream()
        side = self._side_stream() if pipelined else None
        prep_done = [torch.cuda.Event(), torch.cuda.Event()]
        buf_free = [torch.cuda.Event(), torch.cuda.Event()]
        preps: dict[int, dict] = {}

        def proj_ids(c):
            a, b = chunks[c]
            sel = proj[a:b] & (sizes[a:b] > self.small_group)
            return np.arange(a, b, dtype=np.int64)[sel]

        def prep(c):
            ids_c = proj_ids(c)
            if len(ids_c) == 0:
                return
            buf = c % 2
            with torch.cuda.stream(side):
                side.wait_event(buf_free[buf])
                preps[c] = self._prep_projected(fbv, ldp, n_words, gen, grp_first, grp_size, ids_c, sizes, pcnt,
                                                method, buf, xt)
                prep_done[buf].record(side)

        if pipelined:
            start_ev = torch.cuda.Event()
            start_ev.record(main)
            side.wait_event(start_ev)  # the generating level and group tables come from the main stream
            prep(0)
        grp_of = None
        for c, (g0, g1) in enumerate(chunks):
            base = int(offs[g0])
            n_c = int(offs[g1] - base)
            counts = self.scratch.get("chunk_counts", n_c, torch.int32)
            cls = self.scratch.get("chunk_cls", n_c, torch.uint8) if classify else None
            k2_rows = width == 1 and self._k2_rows is not None
            row_wise = k2_rows or k3_rows
            # Fused threshold: the counting kernels set survivor bits (the row-wise kernels count densely and a
            # threshold pass sets the bits after them).
            bits = None
            if self.fused:
                bits = self.scratch.get("chunk_bits", (n_c + 31) // 32 + 1, torch.int32)
                bits.zero_()
            sel = (mc, bits) if (self.fused and not row_wise) else None
            m = sizes[g0:g1]
            ids = np.arange(g0, g1, dtype=np.int64)
            small = m <= self.small_group
            pr = proj[g0:g1]
            # Tile groups too few to fill the GPU (few members over many rows) split their word ranges across
            # CTAs, which add partial counts: the chunk's counts start at zero and its bits come from a
            # threshold pass at the end (the fused kernels leave non-survivors at zero, so the pass agrees).
            tile_ids = ids[~small & ~pr] if not row_wise else ids[:0]
            n_split = 1
            if len(tile_ids):
                nt_t = (sizes[tile_ids] + TILE - 1) // TILE
                n_tp = int((nt_t * (nt_t + 1) // 2).sum())
                n_split = int(max(1, min(-(-n_words // 32), (6 * self._sms()) // max(1, n_tp))))
            if n_split > 1:
                counts.zero_()
            if classify:
                if sel is None:
                    fn = lambda: self.lib.etm_classify(  # noqa: E731
                        _p(gen.rows), width, gen.n, _p(gen.counts), _p(gen.free), _p(grp_first), _p(grp_size),
                        _p(cand_off), g0, g1, mode, _p(cls), _p(counts), _stream())
                else:
                    d2, d3, n_tot = deep if deep is not None else (None, None, n_rows)
                    fn = lambda: self.lib.etm_classify_sel(  # noqa: E731
                        _p(gen.rows), width, gen.n, _p(gen.counts), _p(gen.free), _p(grp_first), _p(grp_size),
                        _p(cand_off), g0, g1, mode if sel is not None else mode & ~4, mc,
                        _p(d2.rows) if d2 is not None else None, d2.n if d2 is not None else 0,
                        _p(d2.counts) if d2 is not None else None, _p(d3.rows) if d3 is not None else None,
                        d3.n if d3 is not None else 0, _p(d3.counts) if d3 is not None else None, n_tot, _p(cls),
                        _p(counts), _p(bits), _stream())
                check(self._launch("classify", n_c * 5, fn), "etm_classify")
                self.launches += 1
                if self.class_stats:
                    by_class = torch.bincount(cls[:n_c].to(torch.int64), minlength=3).cpu().tolist()
                    stats.n_skipped += int(by_class[1])
                    stats.n_inferred += int(by_class[2])
            if k2_rows:
                stats.row_wise = True
                # K=2 from the transactions (one group of every generator): pair counts by row-wise increments.
                rp, cl, nnz, lut, n_r = self._k2_rows
                n_g = int(sizes[0])
                st = self._launch("pair_counts_rows", nnz * 8 + n_r * 8 + n_c * 4, lambda: self.lib.etm_pair_counts_rows(
                    _p(rp), _p(cl), nnz, _p(lut), lut.numel(), n_r, n_g, _p(counts), _stream()))
                check(st, "etm_pair_counts_rows")
                self.launches += 1
            if k3_rows:
                if grp_of is None:
                    grp_of = torch.full((ri["ng"],), -1, dtype=torch.int32, device=self.device)
                    grp_of[gen.rows[grp_first[:G], 0].long()] = torch.arange(G, dtype=torch.int32, device=self.device)
                st = self._launch("triple_counts_rows", ri["nnz"] * 8 + ri["n_r"] * 8 + n_c * 4,
                                  lambda: self.lib.etm_triple_counts_rows(
                                      _p(ri["rp"]), _p(ri["cl"]), ri["nnz"], _p(ri["lut"]), ri["lut"].numel(),
                                      ri["n_r"], _p(gen.rows), _p(grp_of), ri["ng"], _p(grp_first), _p(grp_size),
                                      _p(cand_off), base, n_c, _p(cls), _p(counts), _stream()))
                check(st, "etm_triple_counts_rows")
                self.launches += 2
            for kind, which in (() if (k2_rows or k3_rows) else
                                (("cands", small), ("tiles", ~small & ~pr), ("proj", pr & ~small))):
                gids = ids[which]
                if len(gids) == 0:
                    continue
                if kind == "proj":
                    if pipelined:
                        main.wait_event(prep_done[c % 2])
                        self._count_prepped(preps.pop(c), grp_size, cand_off, base, cls, counts, method, sel)
                        buf_free[c % 2].record(main)
                        continue
                    groups = [gids] if self.form == "batched" else [gids[q:q + 1] for q in range(len(gids))]
                    for bg in groups:
                        self._count_projected(fbv, ldp, n_words, gen, grp_first, grp_size, cand_off, bg, sizes, pcnt,
                                              base, cls, counts, method, sel, xt)
                    continue
                if kind == "tiles" and whole_tc:
                    mg = sizes[gids]
                    toff = np.zeros(len(gids) + 1, np.int64)
                    np.cumsum(_tile_items(mg, 1, self.tc_elem), out=toff[1:])
                    n = len(gids)
                    host = np.concatenate([gids, toff, np.zeros(n, np.int64), np.full(n, n_words, np.int64),
                                           np.full(n, ldp, np.int64)])
                    d = torch.from_numpy(host).to(self.device)
                    self._count_words(fbv, d[2 * n + 1:3 * n + 1], d[3 * n + 1:4 * n + 1], d[4 * n + 1:5 * n + 1],
                                      grp_size, cand_off, d[:n], d[n:2 * n + 1], n, int(toff[-1]), base, cls, counts,
                                      1, int(mg.sum()) * n_words * 8,
                                      float((mg * (mg - 1) / 2).astype(np.float64).sum() * n_rows), sel)
                    continue
                if kind == "cands":
                    w = m[which] * (m[which] - 1) // 2
                else:
                    nt = (m[which] + TILE - 1) // TILE
                    w = nt * (nt + 1) // 2
                batches = [(gids, w)] if self.form == "batched" else [(gids[q:q + 1], w[q:q + 1]) for q in range(len(gids))]
                for bg, bw in batches:
                    wg, wo = self._work(bg, bw)
                    mg = sizes[bg]
                    if kind == "cands":
                        # Every candidate reads its k columns.
                        nbytes = int((mg * (mg - 1) // 2).sum()) * (width + 1) * n_words * 8
                        if sel is None:
                            fn = lambda: self.lib.etm_count_cands(  # noqa: E731
                                _p(fbv), ldp, n_words, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(cand_off),
                                _p(wg), _p(wo), len(bg), base, _p(cls), _p(counts), _stream())
                        else:
                            fn = lambda: self.lib.etm_count_cands_sel(  # noqa: E731
                                _p(fbv), ldp, n_words, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(cand_off),
                                _p(wg), _p(wo), len(bg), base, _p(cls), mc, _p(counts), _p(bits), *self._occ_args(),
                                _stream())
                        st = self._launch("count_cands", nbytes, fn)
                    else:
                        # Each group's prefix and suffix columns, once (the same-data minimum). Groups that reach
                        # this kind under the tensor method hold more than 2^24 rows (past the f32-exact range
                        # of the Gram), so these tiles always count on the CUDA cores.
                        nbytes = int((mg + width - 1).sum()) * n_words * 8
                        if n_split > 1:
                            fn = lambda: self.lib.etm_count_tiles_split(  # noqa: E731
                                _p(fbv), ldp, n_words, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(cand_off),
                                _p(wg), _p(wo), len(bg), int(bw.sum()), base, _p(cls), n_split, _p(counts), _stream())
                        elif sel is None:
                            fn = lambda: self.lib.etm_count_tiles(  # noqa: E731
                                _p(fbv), ldp, n_words, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(cand_off),
                                _p(wg), _p(wo), len(bg), base, _p(cls), 0, _p(counts), _stream())
                        else:
                            fn = lambda: self.lib.etm_count_tiles_sel(  # noqa: E731
                                _p(fbv), ldp, n_words, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(cand_off),
                                _p(wg), _p(wo), len(bg), base, _p(cls), mc, _p(counts), _p(bits), _stream())
                        st = self._launch("count_tiles", nbytes, fn)
                    check(st, f"etm_count_{kind}")
                    self.launches += 1
            if pipelined and c + 1 < len(chunks):
                prep(c + 1)  # overlaps this chunk's counting and the host wait in its compaction
            if self.fused and (row_wise or n_split > 1):
                check(self._launch("threshold_bits", n_c * (5 if classify else 4), lambda: self.lib.etm_threshold_bits(
                    _p(counts), _p(cls), n_c, mc, _p(bits), _stream())), "etm_threshold_bits")
                self.launches += 1
            n_scan = (n_c + 31) // 32 if self.fused else n_c
            ws = self.scratch.get("ws_compact", scan_words(n_scan), torch.int64)
            while True:
                if self.fused:
                    # Reads the bitmask, and the counts of the survivors only.
                    fn = lambda: self.lib.etm_level_compact_bits(  # noqa: E731
                        _p(bits), _p(counts), n_c, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(cand_off),
                        g0, g1, _p(out_rows), _p(out_counts), cap, _p(acc), _p(ws), ws.numel(), _stream())
                    nbytes = (n_c + 7) // 8
                else:
                    fn = lambda: self.lib.etm_level_compact(  # noqa: E731
                        _p(counts), _p(cls), n_c, _p(gen.rows), width, _p(grp_first), _p(grp_size), _p(cand_off), g0,
                        g1, mc, _p(out_rows), _p(out_counts), cap, _p(acc), _p(ws), ws.numel(), _stream())
                    nbytes = n_c * (5 if classify else 4)
                check(self._launch("level_compact", nbytes, fn), "etm_level_compact")
                self.launches += 3
                new_total = int(acc.item())
                if new_total <= cap:
                    break
                # Grow to the level's survivors extrapolated from the candidates counted so far, so that the
                # later chunks compact once.
                done = max(1, int(offs[g1] - offs[0]))
                projected = int(new_total * (total / done) * 1.1)
                cap = int(min(total, max(2 * cap, int(new_total * 1.25), projected)))
                grown_r = torch.empty((cap, width + 1), dtype=torch.int32, device=self.device)
                grown_c = torch.empty(cap, dtype=torch.int32, device=self.device)
                grown_r[:n_out] = out_rows[:n_out]
                grown_c[:n_out] = out_counts[:n_out]
                out_rows, out_counts = grown_r, grown_c
                acc.fill_(n_out)
            n_out = new_total
            stats.n_chunks += 1
        self.check_device_status()
        return Level(out_rows[:n_out], out_counts[:n_out])

    def check_device_status(self) -> None:
        """Raise if a Gram or projection launch since the last check gave up a bounded device wait.

        The kernels record the give-up in device status words instead of hanging; their counts are then
        incomplete, so the level is not returned. The projection's give-up leaves the device in an unknown
        state (bulk copies may still be landing): the caller should stop using the device.
        """
        if not self._waits_pending:
            return
        if self._side is not None:
            torch.cuda.current_stream().wait_stream(self._side)
        self._waits_pending = False
        st = self.lib.etm_device_status(_stream())
        if st != 0:
            raise RuntimeError(f"device counting failed: {self.lib.etm_last_error().decode()}")

    def finish_level(self, new: Level, gen: Level, track_free: bool, prune: bool) -> Level:
        """Free flags against the generating level; under the free-set prune keep the free rows
        whose subsets are all generators (gpu/row_split.py:1075-1100)."""
        if not track_free or new.n == 0:
            if track_free:
                new.free = torch.zeros(0, dtype=torch.uint8, device=self.device)
            return new
        free = torch.empty(new.n, dtype=torch.uint8, device=self.device)
        present = torch.empty(new.n, dtype=torch.uint8, device=self.device) if prune else None
        check(self.lib.etm_level_subsets(_p(new.rows), _p(new.counts), new.n, gen.k, _p(gen.rows), _p(gen.counts),
                                         gen.n, _p(free), _p(present), _stream()), "etm_level_subsets")
        self.launches += 1
        if not prune:
            new.free = free
            return new
        out_r = torch.empty_like(new.rows)
        out_c = torch.empty_like(new.counts)
        out_f = torch.empty_like(free)
        acc = self.scratch.get("acc_sel", 1, torch.int64)
        acc.zero_()
        ws = self.scratch.get("ws_select", scan_words(new.n), torch.int64)
        check(self.lib.etm_select_rows(_p(new.rows), _p(new.counts), _p(free), _p(present), new.n, new.k, _p(out_r),
                                       _p(out_c), _p(free), _p(out_f), new.n, _p(acc), _p(ws), ws.numel(),
                                       _stream()), "etm_select_rows")
        self.launches += 3
        kept = int(acc.item())
        return Level(out_r[:kept], out_c[:kept], out_f[:kept])

    # -- the whole mine ----------------------------------------------------------
    def mine(self, bitvecs, n_rows: int, min_support: float, max_length: int | None = None, *,
             prune_equal_support: bool = False, use_generator_pruning: bool = False,
             level_callback=None, n_cols_logical: int | None = None, rows=None, max_ram_gb: float | None = None,
             max_vram_gb: float | None = None, on_level=None, resume=None, keep_levels: bool = True,
             occupancy: bool = False) -> MineOutput:
        """Mine device bitvectors. ``rows`` = (row_ptr int64, cols int32, host row lengths) on the device,
        the transactions the bitvectors were built from, lets K=2 count row-wise when its rows are short
        against the pair space (the reference's rule, gpu/row_split_chunks.py:124-142). A fourth element
        (int32, -1 for none) makes the entries codes mapped to columns through it; the lengths then count
        only the entries that map to a column.

        ``max_ram_gb`` / ``max_vram_gb``: after every level, the process's resident memory and the device
        memory allocated through torch (every engine buffer) are checked against them; over a limit the mine raises
        MemoryError instead of returning a partial lattice (gpu/row_split.py:467-487).

        ``on_level(k, caller_cols int64 [n, k], counts int64 [n])`` receives every emitted level on the host
        as soon as it is final (the per-level flush); with ``keep_levels=False`` the emitted levels are not kept
        in the output (only the few the next levels need stay on the device).

        ``resume = (k, caller_cols [n, k], counts [n])``: start from a complete emitted level k read back from a
        flush (gpu/row_split.py:546-606): levels 1..k are neither counted nor emitted again; the first resumed
        level has no free flags to infer from, and the deduction bounds wait for levels k-2 and k-3.

        ``occupancy``: build the generating columns' tile occupancy once, and let the prefix and per-candidate
        kernels skip the tiles where a prefix (or a candidate's) column holds no row. It pays when the rows
        are in the input layer's lex order, where deep itemsets' rows gather (gpu/row_split.py:397-413).
        """
        ptr, (n_cols, ld), _owner = as_device_bitvecs(bitvecs)
        self._k2_rows = None
        self._rows_input = None
        self._xt, self._xt_key = None, None  # the row-major copy belongs to one mine's generating columns
        self._occ = None  # so does the tile occupancy
        if n_rows >= 2**31:
            raise ValueError(f"n_transactions={n_rows:,} exceeds int32 max: the count arrays are int32")
        n_words = (n_rows + 63) // 64
        if ld < n_words:
            raise ValueError(f"bitvecs has {ld} words per column, fewer than ceil({n_rows}/64)")
        mc = mining_min_count(min_support, n_rows)
        prune, infer = bool(prune_equal_support), bool(use_generator_pruning) and not prune_equal_support
        track_free = prune or bool(use_generator_pruning)
        t0 = time.perf_counter()
        col_counts = self.column_counts(ptr, n_cols, n_words, ld) if n_cols else np.zeros(0, np.int64)
        freq = np.flatnonzero(col_counts >= mc)
        free1 = col_counts[freq] < n_rows
        gen_cols = freq[free1] if prune else freq
        r_k = int(resume[0]) if resume is not None else 0
        if resume is not None:
            out = MineOutput(n_rows, mc, gen_cols.astype(np.int64), np.zeros(0, np.int64), np.zeros(0, np.int64))
        else:
            out = MineOutput(n_rows, mc, gen_cols.astype(np.int64), gen_cols.astype(np.int64),
                             col_counts[gen_cols].astype(np.int64))
        out.stats.append(LevelStats(1, n_cols, len(gen_cols), (time.perf_counter() - t0) * 1e3))
        #: The level stats of the latest mine (the same list as its MineOutput's).
        self.last_stats = out.stats
        if level_callback and resume is None:
            level_callback(1, n_cols, len(gen_cols), out.stats[-1].ms)
        if on_level is not None and resume is None and len(gen_cols):
            on_level(1, gen_cols[:, None].astype(np.int64), col_counts[gen_cols].astype(np.int64))
        n_logical = n_cols if n_cols_logical is None else n_cols_logical
        max_k = min(max_length if max_length else n_logical, n_logical)
        if len(gen_cols) < 2 or max_k < max(2, r_k + 1):
            return out
        fbv, ldp = self.gather(ptr, ld, gen_cols, n_words)
        ng = len(gen_cols)
        if occupancy:
            self._occ = self.tile_occupancy(fbv, ldp, n_words)
        if rows is not None:
            rp, cl, lens = rows[:3]
            pair_work = float((lens.astype(np.float64) * (lens - 1) / 2).sum())
            lut = torch.full((max(1, n_cols),), -1, dtype=torch.int32, device=self.device)
            lut[torch.from_numpy(gen_cols.astype(np.int64)).to(self.device)] = torch.arange(
                ng, dtype=torch.int32, device=self.device)
            if len(rows) > 3:
                # The entries hold codes and rows[3] their columns (-1 for none): compose code -> generator.
                col_of = rows[3]
                lut = torch.where(col_of >= 0, lut[col_of.clamp(min=0).long()], col_of).contiguous()
            self._rows_input = dict(rp=rp, cl=cl, nnz=int(cl.numel()), lut=lut, n_r=int(rp.numel()) - 1,
                                    pair_work=pair_work, ng=ng)
            r = pair_work / max(1.0, ng * (ng - 1) / 2 * n_words)
            if self.k2_rows_max_r > 0 and r < self.k2_rows_max_r and resume is None:
                self._k2_rows = (rp, cl, int(cl.numel()), lut, int(rp.numel()) - 1)
        if resume is None:
            gen = Level(torch.arange(ng, dtype=torch.int32, device=self.device)[:, None].contiguous(),
                        torch.from_numpy(col_counts[gen_cols].astype(np.int32)).to(self.device),
                        torch.from_numpy(free1[free1] if prune else free1).to(self.device).to(torch.uint8))
            # Complete levels 1, 2, ... (under inference without the free-set prune: every frequent set).
            hist: list[Level | None] = [gen]
            k = 2
        else:
            cols_r = np.asarray(resume[1], np.int64)
            counts_r = np.asarray(resume[2], np.int64)
            gidx = np.searchsorted(gen_cols, cols_r)
            if cols_r.size and (gidx.max() >= ng or (gen_cols[np.minimum(gidx, ng - 1)] != cols_r).any()):
                raise ValueError(f"the level-{r_k} itemsets to resume from hold items that are not frequent here")
            order = np.lexsort(gidx.T[::-1]) if gidx.size else np.zeros(0, np.int64)
            gen = Level(torch.from_numpy(np.ascontiguousarray(gidx[order], dtype=np.int32)).to(self.device),
                        torch.from_numpy(counts_r[order].astype(np.int32)).to(self.device), None)
            hist = [None] * (r_k - 1) + [gen]  # levels 1..k-1 are not at hand: no bounds until three follow
            k = r_k + 1
        while k <= max_k and gen.n >= k:
            t_level = time.perf_counter()
            # Levels k-2 and k-3 for the deduction bounds of level k (k >= 3), when both are at hand.
            d2 = hist[k - 3] if k >= 3 else None
            d3 = hist[k - 4] if k >= 4 else None
            self._deep = (d2, d3, n_rows) if d2 is not None and (k == 3 or d3 is not None) else None
            # The first resumed level has no free flags: inference waits one level.
            level_infer = infer and gen.free is not None
            new, stats = self.count_level(gen, fbv, ldp, n_words, mc, level_infer, prune, n_rows)
            new = self.finish_level(new, gen, track_free, prune)
            stats.n_frequent = new.n
            stats.ms = (time.perf_counter() - t_level) * 1e3
            out.stats.append(stats)
            if level_callback:
                level_callback(k, stats.n_candidates, new.n, stats.ms)
            if max_ram_gb is not None or max_vram_gb is not None:
                check_memory_guard(k, host_rss_gb(), torch.cuda.memory_allocated(self.device) / (1 << 30),
                                   max_ram_gb, max_vram_gb)
            if new.n == 0:
                break
            if on_level is not None:
                on_level(k, out.gen_cols[new.rows.cpu().numpy()], new.counts.cpu().numpy().astype(np.int64))
            if keep_levels:
                out.levels.append(new)
            hist.append(new)
            if len(hist) > 4:
                hist[-5] = None  # the bounds read at most three levels back
            gen = new
            k += 1
        self._deep = None
        self._xt, self._xt_key = None, None
        self._occ = None
        return out


def mine(bitvecs, n_rows: int, min_support: float, max_length: int | None = None, **kw) -> MineOutput:
    """Mine device bitvectors [n_cols, ceil(N/64)] with a fresh ``Engine`` (see ``Engine.mine``)."""
    engine_kw = {k: kw.pop(k) for k in ("method", "form", "chunk_cands", "small_group", "device", "project",
                                        "proj_density", "proj_bytes", "tc_elem", "pipeline", "autotune", "fused",
                                        "deduction_bounds", "proj_rows") if k in kw}
    return Engine(**engine_kw).mine(bitvecs, n_rows, min_support, max_length, **kw)
