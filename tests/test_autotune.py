"""The autotuner's keys, candidate settings and cache persistence (host logic, no GPU)."""

from __future__ import annotations

from importlib import import_module

import numpy as np


def test_keys_bucket_level_shapes(pkg):
    at = import_module(pkg.__name__ + ".autotune").Autotuner()
    a = at.key(3, 31_250, np.array([1200, 800, 5]), 5_000_000_000, "tensor")
    b = at.key(3, 31_000, np.array([1100, 790, 6]), 4_900_000_000, "tensor")
    c = at.key(4, 31_250, np.array([1200, 800, 5]), 5_000_000_000, "tensor")
    assert a == b and a != c


def test_settings_cover_the_knobs(pkg):
    at = import_module(pkg.__name__ + ".autotune").Autotuner()
    assert {s["small_group"] for s in at.settings("tensor")} == set(at.small_groups)
    pop = at.settings("popcount")
    assert len(pop) == len(at.small_groups) * len(at.proj_densities)


def test_cache_round_trip(pkg, tmp_path):
    mod = import_module(pkg.__name__ + ".autotune")
    at = mod.Autotuner()
    at.cache["tensor|k3|w14|med10|max10|c32"] = {"small_group": 64}
    at.save(tmp_path / "tune.json")
    bt = mod.Autotuner()
    bt.load(tmp_path / "tune.json")
    assert bt.cache == at.cache
