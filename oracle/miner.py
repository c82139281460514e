"""CPU oracle: a numpy restatement of ET-Miner's CPU mining route (test infrastructure only).

This module is the oracle the GPU engine is checked against. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it; the engine itself never does, and never falls back to it.

Parity is pinned: ``tests/golden/`` holds results of the reference's own CPU
route (``et_miner.core.cpu_miner._k1_seed`` + ``_mine_levels``), produced by
``tests/golden/make_golden.py``, and ``tests/test_oracle.py`` checks this
module against every one of them.

Each function names the reference code it restates (paths inside the
ET-Miner project). The restatement keeps the algorithm, not the code:

* level K=1 from column counts; free = count < N (``cpu_miner.py:973-981``);
* K=2 pair counts over the generating columns (``count_pairs``,
  ``cpu_miner.py:332-378``; here from bitvectors, which give the same counts);
* K>=3 candidates by prefix join plus the test of the subsets that drop a
  prefix item (``generate_candidates``, ``cpu_miner.py:448-498``);
* Pascal count inference from a non-free (k-1)-subset
  (``cpu_miner.py:1119-1124``);
* counting by AND + popcount of column bitvectors
  (``count_per_candidate``, ``cpu_miner.py:794-809``);
* the free-set test (``_non_free``, ``cpu_miner.py:943-945``, applied at
  ``cpu_miner.py:1139-1151``);
* the level loop (``_mine_levels``, ``cpu_miner.py:1066-1161``).
"""

from __future__ import annotations

import hashlib
import math
from dataclasses import dataclass, field
from fractions import Fraction

import numpy as np


def min_count(min_support: float, n_rows: int) -> int:
    """ceil(s * N) with s read as its shortest round-tripping decimal (``core/result.py:57-79``)."""
    return math.ceil(Fraction(str(min_support)) * n_rows)


def mining_min_count(min_support: float, n_rows: int) -> int:
    """The CPU route's threshold: ``min_count`` but at least 1 (``core/cpu_miner.py:967-970``)."""
    return max(1, min_count(min_support, n_rows))


@dataclass
class CSR:
    """Rows of frequent column ids (ascending per row), the items of the columns, their row counts."""

    indptr: np.ndarray
    cols: np.ndarray
    n_rows: int
    items: np.ndarray
    counts: np.ndarray

    @property
    def n_cols(self) -> int:
        return len(self.items)


def transaction_csr(indptr: np.ndarray, items: np.ndarray, n_rows: int, min_support: float) -> CSR | None:
    """CSR of every row's frequent items (``build_transaction_csr``, ``core/cpu_miner.py:275-308``).

    Items are counted once per row; those reaching ``min_count`` become
    columns in ascending item order; rows map to sorted distinct column ids.
    None when no item is frequent.
    """
    mc = min_count(min_support, n_rows)
    lens = np.diff(indptr)
    rid = np.repeat(np.arange(n_rows, dtype=np.int64), lens)
    # Distinct (row, item) pairs: a repeated item counts once per row.
    key = np.unique(np.stack([rid, items.astype(np.int64)], axis=1), axis=0) if len(items) else np.zeros((0, 2), np.int64)
    uniq_items, counts = np.unique(key[:, 1], return_counts=True) if len(key) else (np.zeros(0, np.int64), np.zeros(0, np.int64))
    keep = counts >= mc
    freq_items = uniq_items[keep]
    if len(freq_items) == 0:
        return None
    col = np.searchsorted(freq_items, key[:, 1])
    col = np.minimum(col, len(freq_items) - 1)
    hit = freq_items[col] == key[:, 1]
    r, c = key[hit, 0], col[hit].astype(np.int32)
    order = np.lexsort((c, r))
    r, c = r[order], c[order]
    out_ptr = np.zeros(n_rows + 1, dtype=np.int64)
    np.cumsum(np.bincount(r, minlength=n_rows), out=out_ptr[1:])
    return CSR(out_ptr, c, n_rows, freq_items, np.bincount(c, minlength=len(freq_items)).astype(np.int64))


def bitvecs_from_csr(indptr: np.ndarray, cols: np.ndarray, n_cols: int, n_rows: int) -> np.ndarray:
    """uint64 [n_cols, ceil(N/64)]: bit r%64 of word r//64 of column c set when row r holds c
    (``build_bitvecs``, ``core/cpu_miner.py:528-578``)."""
    w = (n_rows + 63) // 64
    out = np.zeros(n_cols * w, dtype=np.uint64)
    rows = np.repeat(np.arange(n_rows, dtype=np.int64), np.diff(indptr))
    word = cols.astype(np.int64) * w + (rows >> 6)
    bit = (rows & 63).astype(np.uint64)
    # One OR per bit position: within a position no word repeats.
    for v in range(64):
        sel = bit == v
        if sel.any():
            out[word[sel]] |= np.uint64(1) << np.uint64(v)
    return out.reshape(n_cols, w)


def popcount_rows(a: np.ndarray) -> np.ndarray:
    """Set bits per row of a 2-D uint64 array (``popcount_rows``, ``core/cpu_miner.py:501-505``)."""
    return np.bitwise_count(a).sum(axis=1, dtype=np.int64)


def count_itemsets(sets: np.ndarray, bv: np.ndarray, chunk_bytes: int = 8 << 20) -> np.ndarray:
    """AND of each itemset's columns, popcounted (``count_per_candidate``, ``core/cpu_miner.py:794-809``)."""
    out = np.empty(len(sets), dtype=np.int64)
    step = max(1, chunk_bytes // (8 * max(1, bv.shape[1])))
    for c0 in range(0, len(sets), step):
        c = sets[c0 : c0 + step]
        acc = bv[c[:, 0]].copy()
        for j in range(1, c.shape[1]):
            acc &= bv[c[:, j]]
        out[c0 : c0 + len(c)] = popcount_rows(acc)
    return out


def _pack(rows: np.ndarray, base: int) -> np.ndarray | None:
    """Mixed-radix int64 keys keeping lexicographic order, or None if they could overflow
    (``_pack``, ``core/cpu_miner.py:381-388``)."""
    if rows.shape[1] * math.log2(max(base, 2)) >= 62:
        return None
    key = np.zeros(len(rows), dtype=np.int64)
    for c in range(rows.shape[1]):
        key = key * base + rows[:, c]
    return key


class LevelIndex:
    """Positions of rows in a lexsorted level (``_LevelIndex``, ``core/cpu_miner.py:899-919``)."""

    def __init__(self, level: np.ndarray, base: int):
        self.base = base
        self.keys = _pack(level, base)
        if self.keys is None:
            self.void = np.dtype((np.void, 4 * level.shape[1]))
            rows = np.ascontiguousarray(level, dtype=np.int32).view(self.void).ravel()
            self.order = np.argsort(rows, kind="stable")
            self.sorted = rows[self.order]

    def find(self, sub: np.ndarray) -> np.ndarray:
        if len(sub) == 0:
            return np.zeros(0, dtype=np.int64)
        if self.keys is not None:
            if len(self.keys) == 0:
                return np.full(len(sub), -1, dtype=np.int64)
            key = _pack(sub, self.base)
            pos = np.minimum(np.searchsorted(self.keys, key), len(self.keys) - 1)
            return np.where(self.keys[pos] == key, pos, -1)
        q = np.ascontiguousarray(sub, dtype=np.int32).view(self.void).ravel()
        pos = np.minimum(np.searchsorted(self.sorted, q), len(self.sorted) - 1)
        return np.where(self.sorted[pos] == q, self.order[pos], -1)


def subset_positions(index: LevelIndex, cands: np.ndarray) -> np.ndarray:
    """(n, k) positions of each candidate's (k-1)-subsets; column j drops item j
    (``_Level.subset_positions``, ``core/cpu_miner.py:931-940``)."""
    k = cands.shape[1]
    out = np.empty((len(cands), k), dtype=np.int64)
    for j in range(k):
        out[:, j] = index.find(cands[:, [c for c in range(k) if c != j]])
    return out


def generate_candidates(gen: np.ndarray, k: int, n_cols: int) -> np.ndarray:
    """Lexsorted K-candidates from the lexsorted (k-1)-itemsets ``gen``
    (``generate_candidates``, ``core/cpu_miner.py:448-498``).

    Members of a run of equal first k-2 items pair with every later member;
    a candidate survives when each subset dropping a prefix item is in ``gen``.
    """
    n = len(gen)
    if n < 2:
        return np.zeros((0, k), dtype=np.int32)
    change = np.any(gen[1:, : k - 2] != gen[:-1, : k - 2], axis=1)
    starts = np.flatnonzero(np.r_[True, change])
    sizes = np.diff(np.r_[starts, n])
    pos = np.arange(n) - np.repeat(starts, sizes)
    partners = np.repeat(sizes, sizes) - 1 - pos
    total = int(partners.sum())
    if total == 0:
        return np.zeros((0, k), dtype=np.int32)
    left = np.repeat(np.arange(n, dtype=np.int64), partners)
    right = left + 1 + (np.arange(total, dtype=np.int64) - np.repeat(np.cumsum(partners) - partners, partners))
    cands = np.empty((total, k), dtype=np.int32)
    cands[:, : k - 1] = gen[left]
    cands[:, k - 1] = gen[right, k - 2]
    index = LevelIndex(gen, n_cols)
    keep = np.ones(total, dtype=bool)
    for drop in range(k - 2):
        idx = np.flatnonzero(keep)
        if len(idx) == 0:
            break
        keep[idx] = index.find(cands[idx][:, [c for c in range(k) if c != drop]]) >= 0
    return cands[keep]


@dataclass
class MineResult:
    """Emitted levels as (column-id itemsets lexsorted int32 [n, k], counts int64), plus per-level stats."""

    levels: list[tuple[np.ndarray, np.ndarray]]
    n_rows: int
    min_count: int
    candidates: list[int] = field(default_factory=list)

    def level_sizes(self) -> list[int]:
        return [len(s) for s, _ in self.levels]


def mine_bitvecs(
    bv: np.ndarray,
    n_rows: int,
    min_support: float,
    max_length: int | None = None,
    *,
    prune_equal_support: bool = False,
    use_generator_pruning: bool = False,
) -> MineResult:
    """Frequent itemsets (or free-sets) of column bitvectors ``bv`` [n_cols, ceil(N/64)], column ids in the output.

    The level loop of ``_mine_levels`` (``core/cpu_miner.py:1066-1161``) seeded
    as ``_k1_seed`` (``core/cpu_miner.py:973-981``) seeds it. Columns with a
    count below min_count are not items of the lattice; the threshold is at
    least 1 (``_mining_min_count``).
    """
    n_cols = bv.shape[0]
    mc = mining_min_count(min_support, n_rows)
    col_counts = popcount_rows(bv) if n_cols else np.zeros(0, np.int64)
    freq_cols = np.flatnonzero(col_counts >= mc).astype(np.int32)
    sets1 = freq_cols[:, None]
    counts1 = col_counts[freq_cols]
    free1 = counts1 < n_rows
    gen = sets1[free1] if prune_equal_support else sets1
    res = MineResult([], n_rows, mc, [n_cols])
    res.levels.append((gen, counts1[free1] if prune_equal_support else counts1))
    track_free = prune_equal_support or use_generator_pruning
    infer = use_generator_pruning and not prune_equal_support
    max_k = min(max_length if max_length else n_cols, n_cols)
    # The complete previous level (sets, counts, free flags) the subset lookups resolve against.
    prev_sets, prev_counts, prev_free = sets1, counts1, free1
    k = 2
    while k <= max_k and len(gen) >= k:
        if k == 2:
            g = gen[:, 0]
            ii, jj = np.triu_indices(len(g), 1)
            cands = np.stack([g[ii], g[jj]], axis=1).astype(np.int32)
            counts = count_itemsets(cands, bv) if len(cands) else np.zeros(0, np.int64)
            res.candidates.append(len(cands))
        else:
            cands = generate_candidates(gen, k, n_cols)
            res.candidates.append(len(cands))
            if len(cands) == 0:
                break
            counts = np.empty(len(cands), dtype=np.int64)
            needs = np.ones(len(cands), dtype=bool)
            if infer:
                pos = subset_positions(LevelIndex(prev_sets, n_cols), cands)
                licensed = np.any(~prev_free[pos], axis=1)
                counts[licensed] = prev_counts[pos[licensed]].min(axis=1)
                needs = ~licensed
            if needs.any():
                counts[needs] = count_itemsets(cands[needs], bv)
        keep = counts >= mc
        sets, counts = cands[keep], counts[keep]
        free = None
        if track_free:
            if len(sets):
                pos = subset_positions(LevelIndex(prev_sets, n_cols), sets)
                free = ~np.any(prev_counts[pos] == counts[:, None], axis=1)
            else:
                free = np.zeros(0, dtype=bool)
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
    res.levels = [(s, c) for s, c in res.levels if len(s)]
    return res


def mine_transactions(
    indptr: np.ndarray,
    items: np.ndarray,
    n_rows: int,
    min_support: float,
    max_length: int | None = None,
    *,
    prune_equal_support: bool = False,
    use_generator_pruning: bool = False,
) -> tuple[MineResult, np.ndarray]:
    """The CPU route on a transaction CSR: (result over column ids, the item id of each column)."""
    csr = transaction_csr(indptr, items, n_rows, min_support)
    if csr is None:
        return MineResult([], n_rows, mining_min_count(min_support, n_rows)), np.zeros(0, np.int64)
    bv = bitvecs_from_csr(csr.indptr, csr.cols, csr.n_cols, n_rows)
    res = mine_bitvecs(
        bv, n_rows, min_support, max_length,
        prune_equal_support=prune_equal_support, use_generator_pruning=use_generator_pruning,
    )
    return res, csr.items


def canonical(levels: list[tuple[np.ndarray, np.ndarray]], col_to_item: np.ndarray | None = None) -> list[tuple[tuple[int, ...], int]]:
    """Sorted (itemset of item ids ascending, count) pairs: the comparison form of a result."""
    out = []
    for sets, counts in levels:
        ids = sets if col_to_item is None else col_to_item[sets]
        ids = np.sort(ids, axis=1)
        out += [(tuple(int(v) for v in row), int(c)) for row, c in zip(ids, counts)]
    out.sort(key=lambda t: (len(t[0]), t[0]))
    return out


def digest(levels: list[tuple[np.ndarray, np.ndarray]], col_to_item: np.ndarray | None = None) -> str:
    """SHA-256 over the canonical (k, items..., count) int64 stream, sorted by (k, items)."""
    h = hashlib.sha256()
    per_k: dict[int, list[np.ndarray]] = {}
    for sets, counts in levels:
        if len(sets) == 0:
            continue
        ids = sets if col_to_item is None else np.asarray(col_to_item)[sets]
        ids = np.sort(ids.astype(np.int64), axis=1)
        k = ids.shape[1]
        per_k.setdefault(k, []).append(np.concatenate([ids, np.asarray(counts, np.int64)[:, None]], axis=1))
    for k in sorted(per_k):
        rows = np.concatenate(per_k[k])
        order = np.lexsort(rows[:, :k].T[::-1])
        rows = rows[order]
        head = np.full((len(rows), 1), k, dtype=np.int64)
        h.update(np.ascontiguousarray(np.concatenate([head, rows], axis=1)).astype("<i8").tobytes())
    return h.hexdigest()
