"""etm_level_compact_static: survivor compaction for callers that cannot allocate device memory.

The entry point keeps its scan scratch in an array compiled into the library
instead of taking a workspace from the caller. This test calls it through the
C ABI and checks its output against etm_level_compact (which takes a
caller-allocated workspace) on two calls in a row, exactly (integer results,
zero tolerance). It lives in its own file, collected last, and needs no state
from other tests.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def _level(rng, n_items=120, n_rows=4000):
    """A sorted level of width 2 (distinct pairs a < b) and its prefix groups on the device."""
    import torch

    a = rng.integers(0, n_items, n_rows)
    b = rng.integers(0, n_items, n_rows)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    keep = lo < hi
    rows = np.unique(np.stack([lo[keep], hi[keep]], 1), axis=0).astype(np.int32)
    return torch.from_numpy(rows).cuda(), len(rows)


@pytest.fixture(scope="module")
def setup(pkg):
    import torch

    lib = pkg.load_library()
    rng = np.random.default_rng(2024)
    rows, n = _level(rng)
    gf = torch.empty(n, dtype=torch.int64, device="cuda")
    gs = torch.empty(n, dtype=torch.int32, device="cuda")
    co = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    cnt = torch.empty(2, dtype=torch.int64, device="cuda")
    ws = torch.empty(3 + n // 4096 + 3, dtype=torch.int64, device="cuda")
    st = lib.etm_level_groups(rows.data_ptr(), n, 2, gf.data_ptr(), gs.data_ptr(), co.data_ptr(), cnt.data_ptr(),
                              ws.data_ptr(), ws.numel(), _stream())
    assert st == 0, lib.etm_last_error()
    G, total = (int(x) for x in cnt.cpu().tolist())
    assert G > 10 and total > 10_000
    return lib, rows, gf, gs, co, G, total, rng


def _compact(lib, setup_t, counts, cls, min_count, static: bool):
    import torch

    _, rows, gf, gs, co, G, total, _ = setup_t
    cap = total
    out_rows = torch.full((cap, 3), -1, dtype=torch.int32, device="cuda")
    out_counts = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    acc = torch.zeros(1, dtype=torch.int64, device="cuda")
    cls_p = None if cls is None else cls.data_ptr()
    if static:
        st = lib.etm_level_compact_static(counts.data_ptr(), cls_p, total, rows.data_ptr(), 2, gf.data_ptr(),
                                          gs.data_ptr(), co.data_ptr(), 0, G, min_count, out_rows.data_ptr(),
                                          out_counts.data_ptr(), cap, acc.data_ptr(), _stream())
    else:
        ws = torch.empty(total // 4096 + 3, dtype=torch.int64, device="cuda")
        st = lib.etm_level_compact(counts.data_ptr(), cls_p, total, rows.data_ptr(), 2, gf.data_ptr(), gs.data_ptr(),
                                   co.data_ptr(), 0, G, min_count, out_rows.data_ptr(), out_counts.data_ptr(), cap,
                                   acc.data_ptr(), ws.data_ptr(), ws.numel(), _stream())
    assert st == 0, lib.etm_last_error()
    n = int(acc.item())
    return out_rows[:n].cpu().numpy(), out_counts[:n].cpu().numpy()


def test_static_workspace_matches_workspace_version_twice(setup):
    import torch

    lib, rows, gf, gs, co, G, total, rng = setup
    # Call 1: plain threshold. Call 2: another threshold with a class array (SKIP drops candidates).
    counts1 = torch.from_numpy(rng.integers(0, 1000, total).astype(np.int32)).cuda()
    counts2 = torch.from_numpy(rng.integers(0, 1000, total).astype(np.int32)).cuda()
    cls2 = torch.from_numpy(rng.integers(0, 2, total).astype(np.uint8)).cuda()
    for counts, cls, mc in ((counts1, None, 700), (counts2, cls2, 300)):
        want_rows, want_counts = _compact(lib, setup, counts, cls, mc, static=False)
        got_rows, got_counts = _compact(lib, setup, counts, cls, mc, static=True)
        assert len(want_rows) > 0
        assert np.array_equal(got_rows, want_rows)
        assert np.array_equal(got_counts, want_counts)


def test_static_workspace_rejects_oversized_chunks(setup):
    lib = setup[0]
    too_many = 65536 * 4096 + 1
    st = lib.etm_level_compact_static(None, None, too_many, None, 2, None, None, None, 0, 1, 1, None, None, 0, None,
                                      None)
    assert st == 3  # ETM_ENOSPACE
    assert b"static workspace" in lib.etm_last_error()
