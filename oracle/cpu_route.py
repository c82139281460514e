"""The reference's CPU mining route, restated for timing on the host cores (test infrastructure only).

``oracle/miner.py`` is the parity oracle: it restates *what* the CPU route
computes, counting every candidate by AND + popcount. This module restates
*how* the reference's CPU route counts, so that ``bench.py``'s CPU baseline and
reference arm time the reference's own algorithm on the host cores:

* K=2: every pair count from sparse Gram matrices of the transaction CSR
  (``count_pairs``, ``core/cpu_miner.py:332-378``): column blocks of
  ``M[:, block].T @ M`` (scipy), split by column weight over a thread pool,
  keeping the upper-triangle entries between generating columns that reach
  min_count;
* K>=3: candidates streamed from the previous level in chunks of about
  ``CAND_CHUNK`` (``generate_candidates``, ``cpu_miner.py:448-498``); count
  inference from a non-free subset (``cpu_miner.py:1119-1124``); the rest
  counted one prefix group at a time (``count_candidates``,
  ``cpu_miner.py:727-791``): on column bitvectors of the level's row space
  (rows holding >= k items, ``_level_space`` ``cpu_miner.py:820-832``) when
  they fit ``BITVEC_BUDGET_BYTES`` and the group is small, else as the Gram of
  the suffix columns over the prefix's rows (``gram_pairs``,
  ``cpu_miner.py:641-692``); heavy groups go to the pool;
* the free-set test and the level loop as in ``_mine_levels``
  (``cpu_miner.py:1066-1161``).

The constants are the reference's (``cpu_miner.py:69-93``), so the same input
takes the same path. ``mine`` takes a time budget: when it runs out the mine
stops between blocks or groups and reports how much of each level it counted,
so a bounded run is a measured lower bound of the whole mine's time, never an
extrapolation. Nothing in the engine imports this module.
"""

from __future__ import annotations

import math
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
from scipy.sparse import csc_matrix, csr_matrix

from .miner import bitvecs_from_csr, mining_min_count, popcount_rows

GRAM_BUDGET_BYTES = 256 << 20
CAND_CHUNK = 2_000_000
BITVEC_BUDGET_BYTES = 512 << 20
BITVEC_CHUNK = 125_000
PROJ_MIN_SUFFIXES = ((2048, 40), (float("inf"), 80))
COMPACT_RATIO = 0.5
AND_CHUNK_BYTES = 4 << 20
HEAVY_GROUP_WORK = 2_000_000
PARALLEL_GRAM_WORK = 5_000_000


class Budget:
    """A wall-clock deadline shared by the mine's loops (None: unbounded)."""

    def __init__(self, seconds: float | None):
        self.deadline = None if seconds is None else time.perf_counter() + seconds

    def out(self) -> bool:
        return self.deadline is not None and time.perf_counter() >= self.deadline


def _weighted_ranges(weights: np.ndarray, parts: int, max_width: int) -> list[tuple[int, int]]:
    """Contiguous index ranges of about equal total weight, none wider than ``max_width``."""
    n = len(weights)
    cuts = {0, n}
    total = float(weights.sum()) if n else 0.0
    if total > 0 and parts > 1:
        cum = np.cumsum(weights, dtype=np.float64)
        cuts |= {int(x) for x in np.searchsorted(cum, total * np.arange(1, parts) / parts, side="right")}
    edges = sorted(c for c in cuts if 0 <= c <= n)
    out = []
    for a, b in zip(edges[:-1], edges[1:]):
        out += [(x, min(b, x + max_width)) for x in range(a, b, max_width)]
    return out


def count_pairs(m: csr_matrix, gen: np.ndarray, mc: int, pool, workers: int, budget: Budget):
    """Frequent pairs of generating columns from column blocks of the Gram M.T @ M.

    Returns (pairs int32 [n, 2] lexsorted, counts int64, fraction of the column blocks counted).
    """
    n = m.shape[1]
    if n < 2:
        return np.zeros((0, 2), np.int32), np.zeros(0, np.int64), 1.0
    lens = np.diff(m.indptr).astype(np.int64)
    if pool is not None and int((lens * lens).sum()) < PARALLEL_GRAM_WORK:
        pool, workers = None, 1
    width = max(1, GRAM_BUDGET_BYTES // (12 * n * max(1, workers)))
    parts = 4 * workers if pool is not None else 1
    whole = width >= n and parts == 1
    blocks = [(0, n)] if whole else _weighted_ranges(np.bincount(m.indices, minlength=n), parts, width)
    mt = None if whole else m.T.tocsr()

    def block(rng):
        j0, j1 = rng
        if budget.out():
            return None
        g = (m.T @ m).tocsr() if mt is None else (mt[j0:j1] @ m).tocsr()
        r = np.repeat(np.arange(j0, j1, dtype=np.int32), np.diff(g.indptr))
        c = g.indices
        keep = (c > r) & (g.data >= mc) & gen[r] & gen[c]
        return r[keep], c[keep].astype(np.int32), g.data[keep].astype(np.int64)

    res = list(pool.map(block, blocks)) if pool is not None else [block(b) for b in blocks]
    done = [x for x in res if x is not None]
    frac = len(done) / max(1, len(blocks))
    if not done:
        return np.zeros((0, 2), np.int32), np.zeros(0, np.int64), frac
    i = np.concatenate([d[0] for d in done])
    j = np.concatenate([d[1] for d in done])
    cnt = np.concatenate([d[2] for d in done])
    order = np.lexsort((j, i))
    return np.stack([i[order], j[order]], axis=1), cnt[order], frac


def _entries_of(indptr: np.ndarray, rows: np.ndarray, lens: np.ndarray) -> np.ndarray:
    """Positions in the CSR's indices of every entry of ``rows``, row by row."""
    starts = indptr[rows].astype(np.int64)
    return np.repeat(starts - (np.cumsum(lens) - lens), lens) + np.arange(int(lens.sum()), dtype=np.int64)


def _row_chunks(lens: np.ndarray, chunk: int) -> list[tuple[int, int]]:
    """Consecutive row ranges holding about ``chunk`` entries each."""
    if len(lens) == 0:
        return []
    cum = np.cumsum(lens)
    cuts = [0]
    while cuts[-1] < len(lens):
        base = int(cum[cuts[-1] - 1]) if cuts[-1] else 0
        nxt = int(np.searchsorted(cum, base + chunk, side="right"))
        cuts.append(max(nxt, cuts[-1] + 1))
    cuts[-1] = min(cuts[-1], len(lens))
    return list(zip(cuts[:-1], cuts[1:]))


def gram_pairs(indptr, indices, n_cols, rows, suffix, ia, ib, budget_bytes: int) -> np.ndarray:
    """Counts of the suffix-position pairs (ia < ib) over ``rows``: entries of the Gram of the suffix columns
    over those rows, built in row blocks of G no larger than ``budget_bytes`` and row chunks of about
    ``BITVEC_CHUNK`` entries."""
    out = np.zeros(len(ia), dtype=np.int64)
    if len(ia) == 0:
        return out
    s = len(suffix)
    lut = np.full(n_cols, -1, dtype=np.int32)
    lut[suffix] = np.arange(s, dtype=np.int32)
    lens_all = np.diff(indptr).astype(np.int64)[rows]
    chunks = _row_chunks(lens_all, BITVEC_CHUNK)
    lo, hi = int(ia.min()), int(ia.max()) + 1
    height = max(1, int(budget_bytes // (12 * (s - lo))))
    for a0 in range(lo, hi, height):
        a1 = min(hi, a0 + height)
        sel = np.flatnonzero((ia >= a0) & (ia < a1))
        if len(sel) == 0:
            continue
        g = np.zeros((a1 - a0, s - a0), dtype=np.int64)
        for r0, r1 in chunks:
            lens = lens_all[r0:r1]
            if lens.sum() == 0:
                continue
            pos = lut[indices[_entries_of(indptr, rows[r0:r1], lens)]]
            local = np.repeat(np.arange(r1 - r0, dtype=np.int64), lens)
            keep = pos >= a0
            local, pos = local[keep], pos[keep] - a0
            ptr = np.zeros(r1 - r0 + 1, dtype=np.int64)
            np.cumsum(np.bincount(local, minlength=r1 - r0), out=ptr[1:])
            x = csr_matrix((np.ones(len(pos), dtype=np.int32), pos, ptr), shape=(r1 - r0, s - a0))
            g += (x.T.tocsr()[: a1 - a0] @ x).toarray()
        out[sel] = g[ia[sel] - a0, ib[sel] - a0]
    return out


class RowSpace:
    """The rows a level is counted on (those holding >= k items, or all) and their column bitvectors when they
    fit ``BITVEC_BUDGET_BYTES``; without bitvectors every group is projected over its prefix's rows."""

    def __init__(self, indptr, indices, n_cols, rows=None):
        self.indptr, self.indices, self.n_cols = indptr, indices, n_cols
        self.rows = rows  # ascending transaction ids, or None for every row
        self.n_rows = (len(indptr) - 1) if rows is None else len(rows)
        self.words = (self.n_rows + 63) // 64
        self.bitvecs = None
        if n_cols * self.words * 8 <= BITVEC_BUDGET_BYTES:
            if rows is None:
                self.bitvecs = bitvecs_from_csr(indptr, indices, n_cols, self.n_rows)
            else:
                lens = np.diff(indptr)[rows]
                sub_ptr = np.zeros(len(rows) + 1, np.int64)
                np.cumsum(lens, out=sub_ptr[1:])
                self.bitvecs = bitvecs_from_csr(sub_ptr, indices[_entries_of(indptr, rows, lens)], n_cols,
                                                self.n_rows)
        self.proj_min = next(s for w, s in PROJ_MIN_SUFFIXES if self.words <= w) if self.bitvecs is not None else 0
        self._csc = None

    def full_rows(self, local: np.ndarray) -> np.ndarray:
        return local if self.rows is None else self.rows[local]

    def tidset(self, items: np.ndarray) -> np.ndarray:
        """Transaction ids holding every item (intersection of CSC columns)."""
        if self._csc is None:
            m = csr_matrix((np.ones(len(self.indices), dtype=bool), self.indices, self.indptr),
                           shape=(len(self.indptr) - 1, self.n_cols))
            self._csc = m.tocsc()
        ptr, idx = self._csc.indptr, self._csc.indices
        rows = idx[ptr[items[0]]:ptr[items[0] + 1]]
        for it in items[1:]:
            rows = np.intersect1d(rows, idx[ptr[it]:ptr[it + 1]], assume_unique=True)
        return rows


def level_space(indptr, indices, n_cols, k, space):
    """Rows holding >= k items, rebuilt once they are at most COMPACT_RATIO of the current space."""
    rows_k = np.flatnonzero(np.diff(indptr) >= k)
    if space is None or len(rows_k) <= COMPACT_RATIO * space.n_rows:
        return RowSpace(indptr, indices, n_cols, rows_k if len(rows_k) < len(indptr) - 1 else None)
    return space


def _group_runs(cands: np.ndarray, k: int):
    n = len(cands)
    change = np.any(cands[1:, : k - 2] != cands[:-1, : k - 2], axis=1)
    starts = np.flatnonzero(np.r_[True, change])
    return starts, np.r_[starts[1:], n]


def _count_groups(cands, k, space, starts, ends, out, budget_bytes, budget: Budget, done: list):
    """Per prefix group: AND of the prefix columns, then the pairs counted on bitvectors (small groups) or as
    the Gram over the prefix's rows. Marks each group counted in ``done``."""
    bv = space.bitvecs
    parent_key, parent_and = None, None
    for gi, (s, e) in enumerate(zip(starts.tolist(), ends.tolist())):
        if budget.out():
            return
        prefix = cands[s, : k - 2]
        a, b = cands[s:e, k - 2], cands[s:e, k - 1]
        suffix = np.union1d(a, b)
        ia, ib = np.searchsorted(suffix, a), np.searchsorted(suffix, b)
        if bv is None:
            out[s:e] = gram_pairs(space.indptr, space.indices, space.n_cols, space.tidset(prefix), suffix, ia, ib,
                                  budget_bytes)
        else:
            if k == 3:
                pre = bv[prefix[0]]
            else:
                key = prefix[:-1].tobytes()
                if key != parent_key:
                    parent_key = key
                    parent_and = bv[prefix[0]].copy()
                    for it in prefix[1:-1]:
                        parent_and &= bv[it]
                pre = parent_and & bv[prefix[-1]]
            if len(suffix) >= space.proj_min:
                local = np.flatnonzero(np.unpackbits(pre.view(np.uint8), bitorder="little"))
                out[s:e] = gram_pairs(space.indptr, space.indices, space.n_cols, space.full_rows(local), suffix, ia,
                                      ib, budget_bytes)
            else:
                nz = np.flatnonzero(pre)
                res = np.zeros(e - s, dtype=np.int64)
                if len(nz):
                    sub = bv[suffix[:, None], nz] & pre[nz]
                    step = max(1, AND_CHUNK_BYTES // (8 * len(nz)))
                    for c0 in range(0, e - s, step):
                        c1 = min(c0 + step, e - s)
                        res[c0:c1] = popcount_rows(sub[ia[c0:c1]] & sub[ib[c0:c1]])
                out[s:e] = res
        done.append(e - s)


def count_candidates(cands, k, space, pool, workers, budget: Budget):
    """Counts of lexsorted candidates by prefix group (heavy groups on the pool); returns (counts, counted)
    where counted is the number of candidates whose count was taken before the budget ran out."""
    out = np.full(len(cands), -1, dtype=np.int64)
    starts, ends = _group_runs(cands, k)
    done: list[int] = []
    if pool is None or len(starts) < 2:
        _count_groups(cands, k, space, starts, ends, out, GRAM_BUDGET_BYTES, budget, done)
        return out, sum(done)
    gbytes = GRAM_BUDGET_BYTES // (workers + 1)
    work = (ends - starts).astype(np.float64) * max(1, space.words)
    heavy = work >= HEAVY_GROUP_WORK
    hs, he = starts[heavy], ends[heavy]
    slices = _weighted_ranges(work[heavy], 4 * workers, len(hs)) if len(hs) else []
    futs = [pool.submit(_count_groups, cands, k, space, hs[a:b], he[a:b], out, gbytes, budget, done)
            for a, b in slices]
    _count_groups(cands, k, space, starts[~heavy], ends[~heavy], out, gbytes, budget, done)
    for f in futs:
        f.result()
    return out, sum(done)


class _Members:
    """Which rows of an int32 array are rows of a lexsorted level (packed keys, else void rows)."""

    def __init__(self, level: np.ndarray, base: int):
        self.base = base
        self.keys = None
        if level.shape[1] * math.log2(max(base, 2)) < 62:
            self.keys = self._pack(level)
        else:
            self.void = np.dtype((np.void, 4 * level.shape[1]))
            self.rows = np.sort(np.ascontiguousarray(level, dtype=np.int32).view(self.void).ravel())

    def _pack(self, rows):
        key = np.zeros(len(rows), dtype=np.int64)
        for c in range(rows.shape[1]):
            key = key * self.base + rows[:, c]
        return key

    def contains(self, sub: np.ndarray) -> np.ndarray:
        if self.keys is not None:
            if len(self.keys) == 0:
                return np.zeros(len(sub), dtype=bool)
            key = self._pack(sub)
            pos = np.minimum(np.searchsorted(self.keys, key), len(self.keys) - 1)
            return self.keys[pos] == key
        q = np.ascontiguousarray(sub, dtype=np.int32).view(self.void).ravel()
        pos = np.minimum(np.searchsorted(self.rows, q), len(self.rows) - 1)
        return self.rows[pos] == q


def candidate_chunks(prev: np.ndarray, k: int, n_cols: int):
    """Lexsorted K-candidates of the lexsorted (k-1)-itemsets ``prev`` in chunks of about CAND_CHUNK pairs
    (before the prefix-dropping subset test)."""
    n = len(prev)
    if n < 2:
        return
    change = np.any(prev[1:, : k - 2] != prev[:-1, : k - 2], axis=1)
    starts = np.flatnonzero(np.r_[True, change])
    sizes = np.diff(np.r_[starts, n])
    pos = np.arange(n) - np.repeat(starts, sizes)
    partners = np.repeat(sizes, sizes) - 1 - pos
    cum = np.cumsum(partners)
    member = _Members(prev, n_cols)
    e0 = 0
    while e0 < n:
        before = int(cum[e0 - 1]) if e0 else 0
        e1 = min(max(int(np.searchsorted(cum, before + CAND_CHUNK, side="right")), e0 + 1), n)
        p = partners[e0:e1]
        total = int(p.sum())
        if total:
            left = np.repeat(np.arange(e0, e1, dtype=np.int64), p)
            right = left + 1 + (np.arange(total, dtype=np.int64) - np.repeat(np.cumsum(p) - p, p))
            cands = np.empty((total, k), dtype=np.int32)
            cands[:, : k - 1] = prev[left]
            cands[:, k - 1] = prev[right, k - 2]
            keep = np.ones(total, dtype=bool)
            for drop in range(k - 2):
                idx = np.flatnonzero(keep)
                if len(idx) == 0:
                    break
                keep[idx] = member.contains(cands[idx][:, [c for c in range(k) if c != drop]])
            if keep.any():
                yield cands[keep]
        e0 = e1


@dataclass
class RouteResult:
    """Emitted levels (column ids lexsorted int32 [n, k], counts int64), and what a bounded run completed."""

    levels: list[tuple[np.ndarray, np.ndarray]]
    seconds: float
    complete: bool
    counted: list[dict] = field(default_factory=list)


def mine(indptr: np.ndarray, cols: np.ndarray, n_cols: int, n_rows: int, min_support: float,
         max_length: int | None = None, *, prune_equal_support: bool = False, use_generator_pruning: bool = False,
         workers: int = 1, budget_s: float | None = None) -> RouteResult:
    """The CPU route's mine of a frequent-column CSR (rows of ascending column ids).

    With ``budget_s`` the mine stops when the time runs out (between Gram
    blocks, candidate chunks or prefix groups): ``complete`` is then False and
    ``counted`` says, per level, how many candidates were counted out of how
    many were generated so far. A complete run's levels equal the oracle's.
    """
    t0 = time.perf_counter()
    budget = Budget(budget_s)
    indptr = np.asarray(indptr, np.int64)
    cols = np.asarray(cols, np.int32)
    mc = mining_min_count(min_support, n_rows)
    pool = ThreadPoolExecutor(workers) if workers > 1 else None
    res = RouteResult([], 0.0, True)
    try:
        counts1 = np.bincount(cols, minlength=n_cols).astype(np.int64)
        ones = np.arange(n_cols, dtype=np.int32)[:, None]
        free1 = counts1 < n_rows
        keep1 = counts1 >= mc
        sets1, c1, f1 = ones[keep1], counts1[keep1], free1[keep1]
        gen = sets1[f1] if prune_equal_support else sets1
        res.levels.append((gen, c1[f1] if prune_equal_support else c1))
        res.counted.append({"k": 1, "candidates": n_cols, "counted": n_cols})
        track_free = prune_equal_support or use_generator_pruning
        infer = use_generator_pruning and not prune_equal_support
        prev_sets, prev_counts, prev_free = sets1, c1, f1
        max_tx = int(np.diff(indptr).max()) if n_rows else 0
        max_k = min(max_length if max_length else n_cols, n_cols, max_tx)
        m = csr_matrix((np.ones(len(cols), dtype=np.int32), cols, indptr), shape=(n_rows, n_cols))
        space = None
        k = 2
        while k <= max_k and len(gen) >= k:
            if k == 2:
                gmask = np.zeros(n_cols, dtype=bool)
                gmask[gen[:, 0]] = True
                sets, counts, frac = count_pairs(m, gmask, mc, pool, workers, budget)
                n_c = len(gen) * (len(gen) - 1) // 2
                res.counted.append({"k": 2, "candidates": n_c, "counted": int(round(frac * n_c))})
                if frac < 1.0:
                    res.complete = False
                    break
            else:
                space = level_space(indptr, cols, n_cols, k, space)
                parts_s, parts_c = [], []
                n_c = n_counted = 0
                stopped = False
                for cands in candidate_chunks(gen, k, n_cols):
                    n_c += len(cands)
                    counts = np.empty(len(cands), dtype=np.int64)
                    needs = np.ones(len(cands), dtype=bool)
                    if infer:
                        pos = np.stack([_find(prev_sets, cands[:, [c for c in range(k) if c != j]], n_cols)
                                        for j in range(k)], axis=1)
                        licensed = np.any(~prev_free[pos], axis=1)
                        counts[licensed] = prev_counts[pos[licensed]].min(axis=1)
                        needs = ~licensed
                        n_counted += int(licensed.sum())
                    if needs.any():
                        got, counted = count_candidates(cands[needs], k, space, pool, workers, budget)
                        counts[needs] = got
                        n_counted += counted
                        if counted < int(needs.sum()):
                            stopped = True
                    keep = counts >= mc
                    parts_s.append(cands[keep])
                    parts_c.append(counts[keep])
                    if stopped or budget.out():
                        stopped = True
                        break
                res.counted.append({"k": k, "candidates": n_c, "counted": n_counted, "generated_all": not stopped})
                if stopped:
                    res.complete = False
                    break
                if n_c == 0:
                    break
                sets = np.concatenate(parts_s) if parts_s else np.zeros((0, k), np.int32)
                counts = np.concatenate(parts_c) if parts_c else np.zeros(0, np.int64)
            free = None
            if track_free:
                free = np.zeros(len(sets), dtype=bool)
                if len(sets):
                    pos = np.stack([_find(prev_sets, sets[:, [c for c in range(k) if c != j]], n_cols)
                                    for j in range(k)], axis=1)
                    free = ~np.any(prev_counts[pos] == counts[:, None], axis=1)
            if prune_equal_support:
                gen = sets[free]
                res.levels.append((gen, counts[free]))
            else:
                gen = sets
                res.levels.append((sets, counts))
            prev_sets, prev_counts, prev_free = sets, counts, free
            if len(gen) == 0:
                break
            k += 1
    finally:
        if pool is not None:
            pool.shutdown()
    res.levels = [(s, c) for s, c in res.levels if len(s)]
    res.seconds = time.perf_counter() - t0
    return res


def _find(level: np.ndarray, sub: np.ndarray, base: int) -> np.ndarray:
    """Positions of ``sub``'s rows in the lexsorted ``level`` (every row is present)."""
    if level.shape[1] * math.log2(max(base, 2)) < 62:
        def pack(r):
            key = np.zeros(len(r), dtype=np.int64)
            for c in range(r.shape[1]):
                key = key * base + r[:, c]
            return key
        return np.searchsorted(pack(level), pack(sub))
    void = np.dtype((np.void, 4 * level.shape[1]))
    rows = np.ascontiguousarray(level, dtype=np.int32).view(void).ravel()
    order = np.argsort(rows, kind="stable")
    return order[np.searchsorted(rows[order], np.ascontiguousarray(sub, dtype=np.int32).view(void).ravel())]


def frequent_csr(indptr: np.ndarray, cols: np.ndarray, n_cols: int, n_rows: int, min_support: float):
    """The CSR restricted to the columns reaching min_count, renumbered in ascending order (the CPU route's
    input, ``build_transaction_csr`` ``cpu_miner.py:275-308``): (indptr, cols, kept original column ids)."""
    mc = mining_min_count(min_support, n_rows)
    counts = np.bincount(cols, minlength=n_cols)
    keep = counts >= mc
    remap = np.cumsum(keep) - 1
    sel = keep[cols]
    lens = np.diff(indptr)
    rows = np.repeat(np.arange(n_rows, dtype=np.int64), lens)[sel]
    out_ptr = np.zeros(n_rows + 1, np.int64)
    np.cumsum(np.bincount(rows, minlength=n_rows), out=out_ptr[1:])
    return out_ptr, remap[cols[sel]].astype(np.int32), np.flatnonzero(keep)


def csr_from_column_rows(row_lists: list[np.ndarray], n_rows: int) -> tuple[np.ndarray, np.ndarray]:
    """The row-major CSR (indptr int64, column ids int32) of columns given as ascending row-id lists."""
    lens = np.array([len(r) for r in row_lists], np.int64)
    ptr = np.zeros(len(row_lists) + 1, np.int64)
    np.cumsum(lens, out=ptr[1:])
    idx = np.concatenate(row_lists).astype(np.int32) if len(row_lists) else np.zeros(0, np.int32)
    m = csc_matrix((np.ones(len(idx), dtype=bool), idx, ptr), shape=(n_rows, len(row_lists))).tocsr()
    m.sort_indices()
    return m.indptr.astype(np.int64), m.indices.astype(np.int32)
