"""Host-side planning of the engine, on CPU: projected strides bound the segmented layout, Gram work items per
kernel form, and the row-wise crossover rules."""

from __future__ import annotations

from importlib import import_module

import numpy as np
import pytest


@pytest.fixture(scope="module")
def engm(pkg):
    return import_module(pkg.__name__ + ".engine")


def _padded_words(prefix_rows: np.ndarray, n_words: int, seg: int) -> int:
    """Words of a projected row: per segment of ``seg`` bitvector words, its prefix rows in whole words,
    padded to whole 4-word chunks."""
    n = 0
    for s0 in range(0, n_words * 64, seg * 64):
        c = int(((prefix_rows >= s0) & (prefix_rows < s0 + seg * 64)).sum())
        n += ((c + 63) // 64 + 3) // 4 * 4
    return n


@pytest.mark.parametrize("n_words", [1, 31, 1024, 1025, 5000])
def test_projected_stride_bounds_the_segmented_layout(engm, n_words):
    rng = np.random.default_rng(n_words)
    for density in (0.0, 0.01, 0.3, 1.0):
        rows = np.flatnonzero(rng.random(n_words * 64) < density)
        stride = int(engm.proj_stride(np.array([len(rows)]), n_words)[0])
        used = _padded_words(rows, n_words, engm.PROJ_SEG_WORDS)
        assert used <= stride and stride % 32 == 0 and stride >= 32


def test_gram_items_per_kernel_form(engm):
    m = np.array([1, 2, 240, 241, 256, 257, 512, 1255])
    for elem, t in ((1, 256), (2, 256), (1 | engm.TC_WIDE, 256), (engm.TC_MXF4, 240)):
        nb = (m + t - 1) // t
        assert engm.tc_block(elem) == t
        assert np.array_equal(engm._tile_items(m, 1, elem), nb * (nb + 1) // 2)  # block pairs ua <= ub
    nt = (m + 63) // 64
    assert np.array_equal(engm._tile_items(m, 0), nt * (nt + 1) // 2)  # popcount tile-pairs


def test_row_wise_crossovers_are_the_reference_constants(engm):
    # gpu/row_split_chunks.py:124-159: K2_ROWS_MAX_R and K3_ROWS_MAX_R.
    assert engm.K2_ROWS_MAX_R == 3.95e-3
    assert engm.K3_ROWS_MAX_R == 2.5e-4


def test_memory_guard_raises_past_either_limit(engm):
    """The between-level guard (gpu/row_split.py:467-487): MemoryError naming the level and the limit."""
    import pytest

    engm.check_memory_guard(3, 10.0, 20.0, 800.0, 70.0)
    engm.check_memory_guard(3, 10.0, 20.0, None, None)
    with pytest.raises(MemoryError, match=r"after K=4: RAM=12.0GB exceeds max_ram_gb=8"):
        engm.check_memory_guard(4, 12.0, 1.0, 8.0, 70.0)
    with pytest.raises(MemoryError, match=r"after K=2: VRAM=71.0GB exceeds max_vram_gb=70.0GB.*INCOMPLETE"):
        engm.check_memory_guard(2, 1.0, 71.0, 800.0, 70.0)
    assert engm.host_rss_gb() > 0
