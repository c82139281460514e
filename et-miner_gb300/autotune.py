"""Autotuner for the level driver's counting choices.

A level's candidates can be counted several ways with identical results:
groups of at most ``small_group`` members one warp per candidate, larger ones
by projected tile-pairs (tensor-core Gram or popcount); with the popcount
method a group is projected only when its prefix holds less than
``proj_density`` of the transactions. Which is fastest depends on the level's
shape: the words per column, k, and how the candidates spread over groups.

The tuner keys a level by that shape, bucketed (k, log2 words, log2 of the
median and of the largest group, log2 of the candidate count). The first time
a key appears it counts the level once with every candidate setting, keeps
the fastest (CUDA-event time of the whole level count) and returns that run's
survivors; later levels with the key use the cached setting directly. Levels
below ``min_candidates`` are not tuned (launch overhead dominates). The cache
can be saved to and loaded from JSON so a service tunes once.

This replaces the reference's hand-measured crossover tables
(gpu/row_split_chunks.py:52-121 GROUP_MIN_PAIRS / GROUP_TILED_MIN_PAIRS and
the ET_MINER_* kernel pins), which were fixed per GPU model.
"""

from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np


def _b(x: float) -> int:
    return int(math.floor(math.log2(max(1.0, float(x)))))


@dataclass
class Autotuner:
    """Cache of level shape -> counting settings, filled by timing the candidates."""

    small_groups: tuple[int, ...] = (4, 16, 64)
    proj_densities: tuple[float, ...] = (0.25, 0.5, 1.01)
    min_candidates: int = 1 << 20
    cache: dict[str, dict] = field(default_factory=dict)
    trials: list[dict] = field(default_factory=list)

    def key(self, k: int, n_words: int, sizes: np.ndarray, total: int, method: str) -> str:
        med = float(np.median(sizes)) if len(sizes) else 0.0
        mx = float(sizes.max()) if len(sizes) else 0.0
        return f"{method}|k{k}|w{_b(n_words)}|med{_b(med)}|max{_b(mx)}|c{_b(total)}"

    def settings(self, method: str) -> list[dict]:
        if method == "tensor":
            return [{"small_group": s} for s in self.small_groups]
        return [{"small_group": s, "proj_density": d} for s in self.small_groups for d in self.proj_densities]

    def save(self, path: str | Path) -> None:
        Path(path).write_text(json.dumps(self.cache, indent=1, sort_keys=True))

    def load(self, path: str | Path) -> None:
        p = Path(path)
        if p.exists():
            self.cache.update(json.loads(p.read_text()))
