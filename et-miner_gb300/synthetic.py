"""Seeded synthetic transaction sets for the five mining workloads.

Every generator is deterministic in its seed. Transactions come back as a
CSR: ``indptr`` int64 [n_rows + 1] and ``items`` int64 [nnz], the items of
each row distinct and ascending. The dense K=2 workload (independent
Bernoulli items) is defined by a counter-based hash instead of a random
stream, so the device can produce its bitvectors directly
(``etm_synth_bernoulli``) and this module can produce any slice of the same
bits on the host (``bernoulli_bitvecs``).

Workloads (the item ids, sizes and distributions each one is quoted on):

* ``plain_small``: 60,000 rows over 1,000 ids, Zipf(1.1) popularity, row
  length 1+Poisson(8), drawn without replacement; min_support 0.01.
* ``dense_k2``: 2,000,000 rows x 4,096 items, item i present independently
  with probability p_i ~ Beta(2, 30); min_support 0.002, max_length 3.
* ``deep_sparse``: 20,000,000 rows over 2,000 items; 500 planted patterns
  (length min(1+Poisson(9), 16), Zipf(1.0) items, exponential weights); each
  row of length 1+Poisson(10) is filled from up to four weighted patterns,
  keeping each pattern item with probability 0.7, and padded with uniform
  noise items; min_support 0.005, max_length 16, generator pruning on.
* ``wide_vocab``: 1,000,000 rows over 50,000 items, Zipf(1.0) popularity,
  log-normal lengths (median 8, sigma 1.2) clipped to [1, 500];
  min_support 0.004.
* ``serving``: 8 resident datasets (10K-2M rows, 500-20,000 items,
  Zipf(1.1), 1+Poisson(8) lengths) and 256 requests with Poisson arrivals
  (mean gap 50 ms), log-uniform min_support in [0.002, 0.05] and max_length
  uniform in 2..8.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
ROW_MIX = np.uint64(0xD1B54A32D192ED03)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


@dataclass(frozen=True)
class Transactions:
    """Rows of distinct ascending item ids as a CSR, and the id dtype the workload is quoted with."""

    indptr: np.ndarray
    items: np.ndarray
    n_rows: int

    def row(self, r: int) -> np.ndarray:
        return self.items[self.indptr[r] : self.indptr[r + 1]]

    def rows(self) -> list[list[int]]:
        return [self.row(r).tolist() for r in range(self.n_rows)]


def zipf_weights(n: int, a: float) -> np.ndarray:
    """Popularity of ranks 1..n proportional to rank**-a, normalised."""
    w = np.arange(1, n + 1, dtype=np.float64) ** (-a)
    return w / w.sum()


def _draw_without_replacement(rng: np.random.Generator, weights: np.ndarray, lengths: np.ndarray) -> Transactions:
    """Rows of ``lengths[r]`` distinct items, each drawn by weight among the items not yet in the row.

    Successive weighted draws with repeats rejected are exactly weighted
    sampling without replacement. Each round draws, for every row still
    short, a few more items than it needs; the first occurrence of each
    (row, item) in draw order is kept, then the first ``lengths[r]`` of a row.
    """
    n_items = len(weights)
    lengths = np.minimum(lengths.astype(np.int64), n_items)
    n_rows = len(lengths)
    cdf = np.cumsum(weights)
    cdf /= cdf[-1]
    acc_r = np.zeros(0, dtype=np.int64)
    acc_v = np.zeros(0, dtype=np.int64)
    have = np.zeros(n_rows, dtype=np.int64)
    pending = np.flatnonzero(lengths > 0)
    while len(pending):
        need = lengths[pending] - have[pending]
        rid = np.repeat(pending, need + np.maximum(2, need // 2))
        val = np.minimum(np.searchsorted(cdf, rng.random(len(rid)), side="right"), n_items - 1).astype(np.int64)
        allr = np.concatenate([acc_r, rid])
        allv = np.concatenate([acc_v, val])
        _, first = np.unique(allr * n_items + allv, return_index=True)
        first.sort()
        allr, allv = allr[first], allv[first]
        o = np.argsort(allr, kind="stable")
        allr, allv = allr[o], allv[o]
        c = np.bincount(allr, minlength=n_rows)
        rank = np.arange(len(allr)) - (np.cumsum(c) - c)[allr]
        within = rank < lengths[allr]
        acc_r, acc_v = allr[within], allv[within]
        have = np.bincount(acc_r, minlength=n_rows)
        pending = np.flatnonzero(have < lengths)
    order = np.lexsort((acc_v, acc_r))
    acc_r, acc_v = acc_r[order], acc_v[order]
    indptr = np.zeros(n_rows + 1, dtype=np.int64)
    np.cumsum(np.bincount(acc_r, minlength=n_rows), out=indptr[1:])
    return Transactions(indptr, acc_v, n_rows)


def plain_small(n_rows: int = 60_000, n_items: int = 1_000, seed: int = 0) -> Transactions:
    """60,000 rows over 1,000 ids; Zipf(1.1) popularity; length 1+Poisson(8), no repeats, ascending."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n_items)
    w = np.empty(n_items)
    w[perm] = zipf_weights(n_items, 1.1)
    lengths = 1 + rng.poisson(8, n_rows)
    return _draw_without_replacement(rng, w, lengths)


def wide_vocab(n_rows: int = 1_000_000, n_items: int = 50_000, seed: int = 0) -> Transactions:
    """1M rows over 50,000 ids; Zipf(1.0); log-normal lengths (median 8, sigma 1.2) clipped to [1, 500]."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n_items)
    w = np.empty(n_items)
    w[perm] = zipf_weights(n_items, 1.0)
    lengths = np.clip(np.rint(rng.lognormal(np.log(8.0), 1.2, n_rows)), 1, 500).astype(np.int64)
    return _draw_without_replacement(rng, w, lengths)


def deep_sparse(
    n_rows: int = 20_000_000, n_items: int = 2_000, n_patterns: int = 500, seed: int = 0, patterns_per_row: int = 4
) -> Transactions:
    """Rows filled from planted patterns, then uniform noise (see the module docstring).

    Pattern j has length min(1+Poisson(9), 16), Zipf(1.0) items and weight
    w_j ~ Exponential(1). Row r of length L_r = 1+Poisson(10) draws up to
    ``patterns_per_row`` patterns by weight; each pattern item is kept with
    probability 0.7; the kept items, first occurrence first, fill the row up
    to L_r; uniform noise items pad whatever is left.
    """
    rng = np.random.default_rng(seed)
    plen = np.minimum(1 + rng.poisson(9, n_patterns), 16)
    perm = rng.permutation(n_items)
    wi = np.empty(n_items)
    wi[perm] = zipf_weights(n_items, 1.0)
    pats = _draw_without_replacement(rng, wi, plen)
    pw = rng.exponential(1.0, n_patterns)
    pw /= pw.sum()
    lengths = 1 + rng.poisson(10, n_rows)
    cdf = np.cumsum(pw)
    which = np.minimum(np.searchsorted(cdf, rng.random(n_rows * patterns_per_row), side="right"), n_patterns - 1)
    # Slot order: row-major, so a row's patterns are consecutive and in draw order.
    p_len = np.diff(pats.indptr)[which]
    slot_row = np.repeat(np.arange(n_rows, dtype=np.int64), patterns_per_row)
    rid = np.repeat(slot_row, p_len)
    pos = np.arange(len(rid)) - np.repeat(np.cumsum(p_len) - p_len, p_len)
    val = pats.items[np.repeat(pats.indptr[which], p_len) + pos]
    kept = rng.random(len(rid)) >= 0.3
    rid, val = rid[kept], val[kept]
    rid, val = _first_per_row(rid, val, n_items, lengths)
    have = np.bincount(rid, minlength=n_rows)
    extra = np.maximum(lengths - have, 0)
    while extra.sum() > 0:
        nrid = np.repeat(np.arange(n_rows, dtype=np.int64), extra)
        nval = rng.integers(0, n_items, len(nrid))
        rid, val = _first_per_row(np.concatenate([rid, nrid]), np.concatenate([val, nval]), n_items, lengths)
        extra = np.maximum(lengths - np.bincount(rid, minlength=n_rows), 0)
    order = np.lexsort((val, rid))
    rid, val = rid[order], val[order]
    indptr = np.zeros(n_rows + 1, dtype=np.int64)
    np.cumsum(np.bincount(rid, minlength=n_rows), out=indptr[1:])
    return Transactions(indptr, val.astype(np.int64), n_rows)


@dataclass(frozen=True)
class PatternSpec:
    """Tables of the hash-defined planted-pattern workload (the deep sparse configuration on the device).

    ``len_thr[i]`` = floor(P(1 + Poisson(mean_len) <= i + 1) * 2^64) for i < n_len; ``pat_thr[j]`` =
    floor(cdf_j * 2^64) of the exponential pattern weights; patterns as a CSR (``pat_ptr``, ``pat_items``:
    lengths min(1 + Poisson(9), 16), Zipf(1.0) items without repeats); ``keep_thr`` = floor(0.7 * 2^64).
    """

    len_thr: np.ndarray
    pat_thr: np.ndarray
    pat_ptr: np.ndarray
    pat_items: np.ndarray
    keep_thr: int
    n_items: int
    per_row: int
    hash_seed: int


def _u64_thresholds(cdf: np.ndarray) -> np.ndarray:
    """floor(c * 2^64) of probabilities in [0, 1], exact in integers (1.0 maps to 2^64 - 1)."""
    from math import frexp

    out = np.empty(len(cdf), dtype=np.uint64)
    for i, c in enumerate(np.asarray(cdf, dtype=np.float64).tolist()):
        m, e = frexp(c)  # c = m * 2^e, m in [0.5, 1): floor(c * 2^64) = floor(m * 2^53 * 2^(11 + e))
        mant = int(m * 2**53)
        v = mant << (11 + e) if e >= -11 else mant >> (-(11 + e))
        out[i] = min(v, 2**64 - 1)
    return out


def pattern_spec(n_items: int = 2_000, n_patterns: int = 500, mean_len: float = 10.0, per_row: int = 4,
                 seed: int = 0, hash_seed: int = 777) -> PatternSpec:
    """The deep sparse workload's tables: the same pattern pool, weights and length law as ``deep_sparse``."""
    from math import exp, lgamma, log

    rng = np.random.default_rng(seed)
    plen = np.minimum(1 + rng.poisson(9, n_patterns), 16)
    perm = rng.permutation(n_items)
    wi = np.empty(n_items)
    wi[perm] = zipf_weights(n_items, 1.0)
    pats = _draw_without_replacement(rng, wi, plen)
    pw = rng.exponential(1.0, n_patterns)
    pat_cdf = np.cumsum(pw) / pw.sum()
    # P(Poisson(mean) <= i) for i < 48: the length 1 + Poisson(mean) is capped at 49 (mass past it < 1e-12).
    n_len = 48
    pmf = np.array([exp(i * log(mean_len) - mean_len - lgamma(i + 1)) for i in range(n_len)])
    len_cdf = np.minimum(np.cumsum(pmf), 1.0)
    return PatternSpec(_u64_thresholds(len_cdf), _u64_thresholds(pat_cdf), pats.indptr.astype(np.int64),
                       pats.items.astype(np.int32), int(_u64_thresholds(np.array([0.7]))[0]), n_items, per_row,
                       hash_seed)


def patterns_rows_host(spec: PatternSpec, n_rows: int, row0: int = 0) -> list[list[int]]:
    """Rows ``row0 .. row0 + n_rows - 1`` of the hash-defined pattern workload, each in fill order (the host
    restatement of ``etm_synth_patterns``; a Python loop per row, for small row counts)."""
    seed = spec.hash_seed

    def h(stream: int, r: int) -> int:
        return int(bit_hash(seed, np.array([stream], np.uint64), np.array([r], np.uint64))[0])

    out = []
    for r in range(row0, row0 + n_rows):
        hl = h(1, r)
        length = 1 + sum(1 for t in spec.len_thr if hl >= int(t))
        # The thresholds increase, so counting those reached equals scanning until the first one missed.
        items: list[int] = []
        for p in range(spec.per_row):
            if len(items) >= length:
                break
            hp = h(2 + p, r)
            j = 0
            while j < len(spec.pat_thr) - 1 and hp >= int(spec.pat_thr[j]):
                j += 1
            for q in range(int(spec.pat_ptr[j]), int(spec.pat_ptr[j + 1])):
                if len(items) >= length:
                    break
                if h(64 + 16 * p + (q - int(spec.pat_ptr[j])), r) >= spec.keep_thr:
                    continue
                x = int(spec.pat_items[q])
                if x not in items:
                    items.append(x)
        t = 0
        while len(items) < length and t < 65536:
            x = h(4096 + t, r) % spec.n_items
            t += 1
            if x not in items:
                items.append(x)
        out.append(items)
    return out


def patterns_bitvecs_device(lib, spec: PatternSpec, n_rows: int, device="cuda"):
    """Column bitvectors (torch uint64 [n_items, ceil(n_rows / 64)]) of the pattern workload, built on the
    device by ``etm_synth_patterns``."""
    import torch

    ld = (n_rows + 63) // 64
    t = {k: torch.from_numpy(v).to(device) for k, v in dict(
        len_thr=spec.len_thr.view(np.int64), pat_thr=spec.pat_thr.view(np.int64), pat_ptr=spec.pat_ptr,
        pat_items=spec.pat_items).items()}
    bv = torch.empty((spec.n_items, ld), dtype=torch.int64, device=device)
    st = lib.etm_synth_patterns(t["len_thr"].data_ptr(), len(spec.len_thr), t["pat_thr"].data_ptr(),
                                len(spec.pat_thr), t["pat_ptr"].data_ptr(), t["pat_items"].data_ptr(), spec.per_row,
                                spec.keep_thr, spec.n_items, n_rows, spec.hash_seed, bv.data_ptr(), ld,
                                torch.cuda.current_stream().cuda_stream)
    if st != 0:
        raise RuntimeError(f"etm_synth_patterns failed: {lib.etm_last_error().decode()}")
    return bv.view(torch.uint64)


def _first_per_row(rid: np.ndarray, val: np.ndarray, n_items: int, lengths: np.ndarray):
    """Keep the first occurrence of each (row, item) in the given order, then the first ``lengths[r]`` per row."""
    _, first = np.unique(rid * n_items + val, return_index=True)
    first.sort()
    rid, val = rid[first], val[first]
    o = np.argsort(rid, kind="stable")
    rid, val = rid[o], val[o]
    c = np.bincount(rid, minlength=len(lengths))
    rank = np.arange(len(rid)) - (np.cumsum(c) - c)[rid]
    keep = rank < lengths[rid]
    return rid[keep], val[keep]


def dense_k2_probs(n_items: int = 4_096, seed: int = 0) -> np.ndarray:
    """Per-item presence probabilities p_i ~ Beta(2, 30)."""
    return np.random.default_rng(seed).beta(2.0, 30.0, n_items)


def bernoulli_thresholds(p: np.ndarray) -> np.ndarray:
    """uint64 thresholds: item i is present in row r when hash(seed, i, r) < floor(p_i * 2**64)."""
    return np.floor(np.clip(p, 0.0, 1.0 - 2.0**-53) * 2.0**64).astype(np.uint64)


def bit_hash(seed: int, item: np.ndarray, row: np.ndarray) -> np.ndarray:
    """64-bit counter hash of (seed, item, row): the splitmix64 finaliser of a mixed key."""
    with np.errstate(over="ignore"):
        x = np.uint64(seed) ^ (item.astype(np.uint64) * GOLDEN) ^ (row.astype(np.uint64) * ROW_MIX)
        x = x ^ (x >> np.uint64(30))
        x = x * M1
        x = x ^ (x >> np.uint64(27))
        x = x * M2
        x = x ^ (x >> np.uint64(31))
    return x


def bernoulli_bitvecs(thresholds: np.ndarray, n_rows: int, seed: int) -> np.ndarray:
    """Column bitvectors uint64 [n_items, ceil(n_rows / 64)] of the hash-defined Bernoulli workload (host twin)."""
    n_items = len(thresholds)
    w = (n_rows + 63) // 64
    out = np.zeros((n_items, w), dtype=np.uint64)
    rows = np.arange(n_rows, dtype=np.uint64)
    for i in range(n_items):
        bits = bit_hash(seed, np.full(n_rows, i, dtype=np.uint64), rows) < thresholds[i]
        padded = np.zeros(w * 64, dtype=bool)
        padded[:n_rows] = bits
        out[i] = np.packbits(padded.reshape(w, 64), axis=1, bitorder="little").view(np.uint64)[:, 0]
    return out


def bitvecs_to_transactions(bv: np.ndarray, n_rows: int) -> Transactions:
    """The CSR of the rows a column-bitvector array describes (bit r % 64 of word r // 64 of column c)."""
    n_cols = bv.shape[0]
    bits = np.unpackbits(np.ascontiguousarray(bv).view(np.uint8), axis=1, bitorder="little")[:, :n_rows]
    cols, rows = np.nonzero(bits)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    indptr = np.zeros(n_rows + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n_rows), out=indptr[1:])
    del n_cols
    return Transactions(indptr, cols.astype(np.int64), n_rows)


@dataclass(frozen=True)
class Request:
    """One serving request: which resident dataset, its thresholds, and when it arrives (seconds from start)."""

    dataset: int
    min_support: float
    max_length: int
    arrival_s: float


def serving_datasets(seed: int = 0, scale: float = 1.0) -> list[tuple[Transactions, int]]:
    """Eight resident datasets, 10K-2M rows (times ``scale``) and 500-20,000 items: (transactions, n_items)."""
    rng = np.random.default_rng(seed)
    rows = np.geomspace(10_000, 2_000_000, 8)
    items = np.geomspace(500, 20_000, 8)
    order = rng.permutation(8)
    out = []
    for d in range(8):
        n_rows = max(64, int(rows[d] * scale))
        n_items = int(items[order[d]])
        t = _serving_rows(n_rows, n_items, int(rng.integers(1 << 31)))
        out.append((t, n_items))
    return out


def _serving_rows(n_rows: int, n_items: int, seed: int) -> Transactions:
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n_items)
    w = np.empty(n_items)
    w[perm] = zipf_weights(n_items, 1.1)
    return _draw_without_replacement(rng, w, 1 + rng.poisson(8, n_rows))


def serving_requests(n: int = 256, mean_gap_s: float = 0.05, seed: int = 0) -> list[Request]:
    """``n`` requests with exponential inter-arrival gaps, uniform dataset choice,
    log-uniform min_support in [0.002, 0.05] and max_length uniform in 2..8."""
    rng = np.random.default_rng(seed + 1)
    t = np.cumsum(rng.exponential(mean_gap_s, n))
    ds = rng.integers(0, 8, n)
    s = np.exp(rng.uniform(np.log(0.002), np.log(0.05), n))
    ml = rng.integers(2, 9, n)
    return [Request(int(ds[i]), float(s[i]), int(ml[i]), float(t[i])) for i in range(n)]
