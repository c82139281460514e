"""Size-independent checks of a mine result against counts recomputed in plain PyTorch.

A mine of a full-size workload cannot be compared with a CPU mine of the same
input (the CPU route would take hours), so its result is checked by
properties that hold at any size, with every count recomputed independently
of the engine's kernels: an AND of the itemset's column words and a SWAR
popcount, both plain PyTorch tensor ops on the caller's bitvectors.

* exact counts: a sample of every emitted level is recounted;
* level 1 complete: every column reaching min_count is emitted (under the
  free-set prune: every such column with count < N);
* closure: every (k-1)-subset of a sampled itemset is emitted with a count at
  least as large (frequent itemsets, and generators, are closed under
  subsets);
* completeness and absence: a sampled itemset of level k-1 extended by a
  random larger frequent item is recounted; it must be emitted, with that
  count, exactly when it is frequent (and, under the free-set prune, free
  with every subset emitted), and absent otherwise.

This is the reference's full-lattice gate (tests/test_tier_equivalence.py:
176-245) restated for inputs the oracle cannot mine: the sample stands in for
the whole lattice.
"""

from __future__ import annotations

import numpy as np
import torch

from .engine import MineOutput

_M1 = 0x5555555555555555
_M2 = 0x3333333333333333
_M4 = 0x0F0F0F0F0F0F0F0F
_H01 = 0x0101010101010101


def popcount64(x: torch.Tensor) -> torch.Tensor:
    """Set bits of every int64 element (SWAR; the arithmetic shifts are masked, so the sign does not leak)."""
    x = x - ((x >> 1) & _M1)
    x = (x & _M2) + ((x >> 2) & _M2)
    x = (x + (x >> 4)) & _M4
    return ((x * _H01) >> 56) & 0xFF


class Recount:
    """Support counts of column sets over device bitvectors (int64 view [n_cols, W]), in plain PyTorch."""

    def __init__(self, bv: torch.Tensor, batch_bytes: int = 256 << 20):
        self.bv = bv.view(torch.int64) if bv.dtype != torch.int64 else bv
        self.batch = max(1, batch_bytes // (8 * max(1, self.bv.shape[1])))

    def __call__(self, sets: torch.Tensor) -> torch.Tensor:
        """Counts (int64 [n]) of the itemsets ``sets`` (int64 [n, k] caller column ids)."""
        out = []
        for b0 in range(0, sets.shape[0], self.batch):
            s = sets[b0:b0 + self.batch]
            acc = self.bv[s[:, 0]].clone()
            for c in range(1, s.shape[1]):
                acc &= self.bv[s[:, c]]
            out.append(popcount64(acc).sum(dim=1))
        return torch.cat(out) if out else torch.zeros(0, dtype=torch.int64, device=self.bv.device)

    def columns(self) -> torch.Tensor:
        return torch.cat([popcount64(self.bv[c0:c0 + self.batch]).sum(dim=1)
                          for c0 in range(0, self.bv.shape[0], self.batch)])


class _LevelIndex:
    """Membership and counts of the rows of one level (int64 [n, k] caller columns) on the device: rows are
    keyed by a 64-bit polynomial hash, sorted; a hit is confirmed by comparing the row itself."""

    MUL = 0x100000001B3

    def __init__(self, rows: torch.Tensor, counts: torch.Tensor):
        self.rows, self.counts = rows, counts
        self.keys, self.order = torch.sort(self._hash(rows))

    @classmethod
    def _hash(cls, rows: torch.Tensor) -> torch.Tensor:
        h = torch.full((rows.shape[0],), 0x2545F4914F6CDD1D, dtype=torch.int64, device=rows.device)
        for c in range(rows.shape[1]):
            h = (h ^ rows[:, c]) * cls.MUL  # wraps modulo 2^64
        return h

    def find(self, q: torch.Tensor) -> torch.Tensor:
        """Position of each query row in ``rows``, or -1."""
        if self.rows.shape[0] == 0:
            return torch.full((q.shape[0],), -1, dtype=torch.int64, device=q.device)
        h = self._hash(q)
        pos = torch.searchsorted(self.keys, h).clamp(max=len(self.keys) - 1)
        # Equal hashes are adjacent after the sort; scan a few neighbours for the exact row.
        found = torch.full((q.shape[0],), -1, dtype=torch.int64, device=q.device)
        for d in range(4):
            p = (pos + d).clamp(max=len(self.keys) - 1)
            cand = self.order[p]
            hit = (self.keys[p] == h) & (self.rows[cand] == q).all(dim=1) & (found < 0)
            found = torch.where(hit, cand, found)
        return found


def check_mine(out: MineOutput, bv: torch.Tensor, n_rows: int, *, prune: bool = False, generators: bool = False,
               max_length: int | None = None, sample: int = 10_000, seed: int = 0) -> dict:
    """Check a mine of ``bv`` (the caller's bitvectors, uint64/int64 [n_cols, W] on the device).

    ``prune`` / ``generators``: the mine ran with prune_equal_support / use_generator_pruning (the latter
    changes no emitted itemset, only how counts are obtained). Returns the numbers checked and the
    mismatches found (all zero when the result is right).
    """
    dev = bv.device
    recount = Recount(bv)
    mc = out.min_count
    gen = torch.from_numpy(out.gen_cols.astype(np.int64)).to(dev)
    rng = torch.Generator(device="cpu").manual_seed(seed)
    rep = {"min_count": mc, "levels": [], "count_mismatches": 0, "closure_violations": 0,
           "extension_mismatches": 0, "sampled": 0, "extensions_checked": 0, "extensions_frequent": 0}

    # Level 1.
    pc = recount.columns()
    want1 = (pc >= mc) & ((pc < n_rows) if prune else torch.ones_like(pc, dtype=torch.bool))
    l1 = torch.from_numpy(out.level1_cols.astype(np.int64)).to(dev)
    got1 = torch.zeros_like(want1)
    got1[l1] = True
    rep["level1_complete"] = bool(torch.equal(got1, want1))
    rep["level1_counts_exact"] = bool(torch.equal(pc[l1], torch.from_numpy(out.level1_counts).to(dev)))
    levels = [(l1[:, None], torch.from_numpy(out.level1_counts.astype(np.int64)).to(dev))]
    for lv in out.levels:
        if lv.n:
            levels.append((gen[lv.rows.long()], lv.counts.long()))
    index = [_LevelIndex(r, c) for r, c in levels]
    freq_items = torch.nonzero(pc >= mc).flatten()

    for li, (rows, counts) in enumerate(levels):
        k = rows.shape[1]
        n = rows.shape[0]
        pick = torch.randperm(n, generator=rng)[:sample].to(dev)
        s_rows, s_counts = rows[pick], counts[pick]
        # Exact counts.
        mism = int((recount(s_rows) != s_counts).sum()) if k > 1 else 0
        # Closure.
        viol = 0
        if k > 1:
            for d in range(k):
                sub = torch.cat([s_rows[:, :d], s_rows[:, d + 1:]], dim=1)
                p = index[li - 1].find(sub)
                ok = (p >= 0)
                ok &= torch.where(p >= 0, index[li - 1].counts[p.clamp(min=0)] >= s_counts, ok)
                viol += int((~ok).sum())
        # Extensions by a larger frequent item.
        ext_checked = ext_freq = ext_bad = 0
        if max_length is None or k + 1 <= max_length:
            last = s_rows[:, -1].contiguous()
            u = torch.rand(len(pick), generator=rng).to(dev)
            lo = torch.searchsorted(freq_items, last, right=True)
            n_larger = len(freq_items) - lo
            has = n_larger > 0
            if has.any():
                off = torch.minimum((u * n_larger).long(), (n_larger - 1).clamp(min=0))
                y = freq_items[(lo + off)[has]]
                base = s_rows[has]
                cand = torch.cat([base, y[:, None]], dim=1)
                cnt = recount(cand)
                frequent = cnt >= mc
                expect = frequent.clone()
                if prune:
                    # Emitted only when every k-subset is emitted with a larger count (free, and a generator);
                    # under generator pruning alone every frequent itemset is emitted (the pruning only infers
                    # counts).
                    for d in range(k + 1):
                        sub = torch.cat([cand[:, :d], cand[:, d + 1:]], dim=1)
                        p = index[li].find(sub)
                        subc = torch.where(p >= 0, index[li].counts[p.clamp(min=0)], torch.zeros_like(p))
                        expect &= (p >= 0) & (subc > cnt)
                if li + 1 < len(index):
                    p = index[li + 1].find(cand)
                    present = p >= 0
                    same = torch.where(present, index[li + 1].counts[p.clamp(min=0)] == cnt, present)
                else:
                    present = torch.zeros_like(expect)
                    same = present
                ext_bad = int((present != expect).sum() + (present & ~same).sum())
                ext_checked = int(len(cand))
                ext_freq = int(frequent.sum())
        rep["levels"].append({"k": k, "emitted": n, "sampled": int(len(pick)), "count_mismatches": mism,
                              "closure_violations": viol, "extensions": ext_checked,
                              "extensions_frequent": ext_freq, "extension_mismatches": ext_bad})
        rep["count_mismatches"] += mism
        rep["closure_violations"] += viol
        rep["extension_mismatches"] += ext_bad
        rep["sampled"] += int(len(pick))
        rep["extensions_checked"] += ext_checked
        rep["extensions_frequent"] += ext_freq
    rep["mismatches"] = (rep["count_mismatches"] + rep["closure_violations"] + rep["extension_mismatches"]
                         + (0 if rep["level1_complete"] and rep["level1_counts_exact"] else 1))
    return rep
