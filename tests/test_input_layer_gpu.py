"""GPU parity of the input layer's lex row order and the tile-occupancy skip.

The row order keys, the row permutation and the tile occupancy are checked word for word against host
restatements; mining with the occupancy skip, and through the transactions route in lex order, must give
exactly the itemsets and counts of the same mine without them.
"""

from __future__ import annotations

from importlib import import_module

import numpy as np
import pytest

from tests.helpers import table_of

pytestmark = pytest.mark.gpu

TOP = np.uint64(1 << 63)


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def _host_keys(rp: np.ndarray, cols: np.ndarray, rank: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The lex order keys (gpu/kernels/_src/csr_to_bitvec.cu:75-104) as unsigned values."""
    n = len(rp) - 1
    hi = np.zeros(n, np.uint64)
    lo = np.zeros(n, np.uint64)
    for r in range(n):
        for c in cols[rp[r]:rp[r + 1]]:
            k = int(rank[c])
            if k < 64:
                hi[r] |= np.uint64(1) << np.uint64(63 - k)
            elif k < 128:
                lo[r] |= np.uint64(1) << np.uint64(127 - k)
    return hi, lo


def _random_csr(rng, n_rows: int, n_cols: int, max_len: int):
    lens = rng.integers(0, max_len + 1, n_rows)
    lens[::29] = 0
    rp = np.zeros(n_rows + 1, np.int64)
    np.cumsum(lens, out=rp[1:])
    cols = np.concatenate([np.sort(rng.choice(n_cols, size=int(k), replace=False)) for k in lens]).astype(np.int32) \
        if lens.sum() else np.zeros(0, np.int32)
    return rp, cols


@pytest.mark.parametrize("n_cols,max_len", [(40, 30), (200, 30), (300, 150)])
def test_row_order_keys_and_permutation(pkg, n_cols, max_len):
    """Rows of up to 150 entries take several warp-wide steps per row."""
    import torch

    api = import_module(pkg.__name__ + ".api")
    lib = pkg.load_library()
    rng = np.random.default_rng(n_cols)
    n_rows = 3_001
    rp, cols = _random_csr(rng, n_rows, n_cols, max_len)
    support = np.bincount(cols, minlength=n_cols)
    rank = np.empty(n_cols, np.int32)
    rank[np.argsort(-support, kind="stable")] = np.arange(n_cols, dtype=np.int32)
    rp_d = torch.from_numpy(rp).cuda()
    cols_d = torch.from_numpy(cols).cuda()
    key_hi = torch.empty(n_rows, dtype=torch.int64, device="cuda")
    key_lo = torch.empty(n_rows, dtype=torch.int64, device="cuda")
    st = lib.etm_row_order_keys(rp_d.data_ptr(), cols_d.data_ptr(), n_rows, torch.from_numpy(rank).cuda().data_ptr(),
                                n_cols, key_hi.data_ptr(), key_lo.data_ptr(), _stream())
    assert st == 0, lib.etm_last_error()
    hi, lo = _host_keys(rp, cols, rank)
    assert np.array_equal(key_hi.cpu().numpy().view(np.uint64) ^ TOP, hi)
    assert np.array_equal(key_lo.cpu().numpy().view(np.uint64) ^ TOP, lo)

    new_rp, new_cols, new_len = api._lex_order(rp_d, cols_d, support)
    order = np.lexsort((lo, hi))  # stable: by (hi, lo) ascending, ties in input order
    want_len = np.diff(rp)[order]
    assert np.array_equal(new_len, want_len)
    assert np.array_equal(new_rp.cpu().numpy()[1:], np.cumsum(want_len))
    want_cols = np.concatenate([cols[rp[r]:rp[r + 1]] for r in order])
    assert np.array_equal(new_cols.cpu().numpy(), want_cols)


def test_permute_rows_refuses_a_bad_order(pkg):
    """An order entry outside [0, n_rows) is skipped on the device and reported, not followed."""
    import torch

    lib = pkg.load_library()
    rp = torch.tensor([0, 2, 3, 5], dtype=torch.int64, device="cuda")
    cols = torch.tensor([1, 4, 2, 0, 3], dtype=torch.int32, device="cuda")
    order = torch.tensor([2, 7, 0], dtype=torch.int64, device="cuda")
    new_rp = torch.tensor([0, 2, 3, 5], dtype=torch.int64, device="cuda")
    out = torch.full((5,), -1, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = lib.etm_permute_rows(rp.data_ptr(), cols.data_ptr(), 5, order.data_ptr(), 3, new_rp.data_ptr(),
                              out.data_ptr(), status.data_ptr(), _stream())
    assert st == 0, lib.etm_last_error()
    assert int(status.item()) == 1
    assert out.cpu().tolist() == [0, 3, -1, 1, 4]


@pytest.mark.parametrize("n_words", [1, 31, 32, 33, 2_047, 2_048, 2_049, 5_000])
@pytest.mark.parametrize("odd_ld", [False, True])
def test_tile_occupancy_matches_host(pkg, n_words, odd_ld):
    """Padded columns (16-byte loads) and the reference's own layout, ld = the words per column (8-byte loads
    where a column starts off a 16-byte boundary)."""
    import torch

    lib = pkg.load_library()
    rng = np.random.default_rng(n_words)
    n_cols = 7
    ld = n_words + (n_words % 2) + 2
    if odd_ld:
        ld = n_words + 1 - (n_words % 2)
    bv = np.zeros((n_cols, ld), np.uint64)
    for c in range(n_cols):
        # A few words set per column, some columns empty, garbage past n_words that must be ignored.
        if c % 3 == 2:
            continue
        at = rng.choice(n_words, size=max(1, n_words // (50 * (c + 1))), replace=False)
        bv[c, at] = rng.integers(1, 2**63, len(at)).astype(np.uint64)
    bv[:, n_words:] = np.uint64(0xFFFF)
    tiles = -(-n_words // 32)
    occ_ld = -(-tiles // 64) + 1
    occ = torch.full((n_cols, occ_ld), -1, dtype=torch.int64, device="cuda")
    d = torch.from_numpy(bv.view(np.int64)).cuda()
    st = lib.etm_tile_occupancy(d.data_ptr(), n_cols, n_words, ld, occ.data_ptr(), occ_ld, _stream())
    assert st == 0, lib.etm_last_error()
    want = np.zeros((n_cols, occ_ld), np.uint64)
    for c in range(n_cols):
        for t in range(64 * occ_ld):
            lo, hi = 32 * t, min(n_words, 32 * t + 32)
            if lo < hi and (bv[c, lo:hi] != 0).any():
                want[c, t // 64] |= np.uint64(1) << np.uint64(t % 64)
    assert np.array_equal(occ.cpu().numpy().view(np.uint64), want)
    assert lib.etm_tile_occupancy(d.data_ptr(), n_cols, n_words, ld, occ.data_ptr(), 0, _stream()) == 1


def _topic_bitvecs(n_rows: int, seed: int):
    """Rows in blocks of 4,096, block b on topic b % 10: the topic's 12 items at 0.5 each in its rows, one wide
    topic (40 items at 0.45) on every fourth block, and 4 items at 0.05 everywhere. Most 32-word tiles hold no
    row of a topic item, so the occupancy skips most of them."""
    rng = np.random.default_rng(seed)
    n_items = 10 * 12 + 40 + 4
    dense = np.zeros((n_rows, n_items), bool)
    for b0 in range(0, n_rows, 4096):
        b = b0 // 4096
        r = slice(b0, min(n_rows, b0 + 4096))
        n = r.stop - r.start
        t = b % 10
        dense[r, 12 * t:12 * t + 12] = rng.random((n, 12)) < 0.5
        if b % 4 == 0:
            dense[r, 120:160] = rng.random((n, 40)) < 0.45
    dense[:, 160:] = rng.random((n_rows, 4)) < 0.05
    n_words = -(-n_rows // 64)
    bits = np.packbits(dense.T, axis=1, bitorder="little")
    pad = np.zeros((n_items, n_words * 8), np.uint8)
    pad[:, :bits.shape[1]] = bits
    return pad.view(np.uint64), n_items


@pytest.mark.parametrize("form", ["batched", "popcount", "plain", "proj", "proj_cols"])
def test_occupancy_skip_leaves_counts_unchanged(pkg, form):
    import torch

    engm = import_module(pkg.__name__ + ".engine")
    kw = {"batched": {}, "popcount": dict(method="popcount"), "plain": dict(form="plain"),
          "proj": dict(small_group=2, proj_density=1.01, proj_bytes=1 << 16),
          "proj_cols": dict(small_group=2, proj_density=1.01, proj_bytes=1 << 16, proj_rows=False)}[form]
    bv, n_items = _topic_bitvecs(150_000, 3)
    dev = torch.from_numpy(bv.view(np.int64)).cuda().view(torch.uint64)
    res = []
    for occ in (False, True):
        eng = engm.Engine(**kw)
        eng.profile_kernels = True
        out = eng.mine(dev, 150_000, 0.003, 4, occupancy=occ)
        res.append(out.host_levels())
        if occ:
            assert "tile_occupancy" in eng.kernel_report()
    a, b = res
    assert len(a) == len(b) >= 3
    for (ra, ca), (rb, cb) in zip(a, b):
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb)


def test_transactions_in_lex_order_match_input_order(pkg):
    """apriori(transactions): the lex row order with the occupancy skip against the rows in input order."""
    engm = import_module(pkg.__name__ + ".engine")
    bv, n_items = _topic_bitvecs(60_000, 11)
    dense = np.unpackbits(bv.view(np.uint8), axis=1, bitorder="little")[:, :60_000].T.astype(bool)
    rows_i, cols_i = np.nonzero(dense)
    indptr = np.zeros(60_001, np.int64)
    np.cumsum(np.bincount(rows_i, minlength=60_000), out=indptr[1:])
    items = (cols_i * 7 + 3).astype(np.int64)  # ids that are not the columns
    got = []
    for order in ("lex", "keep"):
        eng = engm.Engine()
        eng.row_order, eng.lex_min_rows = order, 0
        df = pkg.apriori(table_of(indptr, items, 60_000), min_support=0.004, max_length=4, use_gpu=True, engine=eng,
                         warn_complexity=False)
        got.append(pkg.result_pairs(df, 60_000))
    assert got[0] == got[1]
    assert max(len(s) for s, _ in got[0]) == 4


def _canonical_csr(rng, n_rows: int, ids: np.ndarray, max_len: int):
    lens = rng.integers(0, max_len + 1, n_rows)
    lens[::31] = 0
    rp = np.zeros(n_rows + 1, np.int64)
    np.cumsum(lens, out=rp[1:])
    flat = np.concatenate([np.sort(rng.choice(ids, size=int(k), replace=False)) for k in lens]) if lens.sum() \
        else np.zeros(0, np.int64)
    return rp, flat.astype(np.int64)


@pytest.mark.parametrize("mc,max_len", [(1, 25), (40, 25), (40, 200)])
def test_coded_input_matches_host(pkg, mc, max_len):
    """The sort-free coding gives the columns, supports and rows of the host restatement (rows of up to 200
    ids take several warp-wide steps, and the canonical check carries across them)."""
    import torch

    api = import_module(pkg.__name__ + ".api")
    rng = np.random.default_rng(mc + max_len)
    ids = np.unique(rng.integers(-5_000, 90_000, 300 if max_len < 100 else 600))
    n_rows = 4_000
    rp, flat = _canonical_csr(rng, n_rows, ids, max_len)
    rp_h, cols_h, items_h = api._frequent_csr(rp, flat, n_rows, mc)
    got = api._coded_csr_device(rp, flat, n_rows, mc, torch.device("cuda"))
    assert got is not None
    assert np.array_equal(got.items, items_h)
    assert np.array_equal(got.support, np.bincount(cols_h, minlength=len(items_h)))
    assert np.array_equal(got.row_len, np.diff(rp_h))
    cols = got.col_of[got.codes.long()].cpu().numpy()
    assert np.array_equal(cols[cols >= 0], cols_h)
    assert np.array_equal(got.row_ptr.cpu().numpy(), rp)
    assert len(got.code_support) == len(np.unique(flat))


def test_coded_input_with_more_ids_than_shared_counters(pkg):
    """More distinct ids than the histogram's block-private counters hold: the global-atomic form."""
    import torch

    api = import_module(pkg.__name__ + ".api")
    rng = np.random.default_rng(5)
    ids = np.unique(rng.integers(0, 400_000, 30_000))
    n_rows = 20_000
    rp, flat = _canonical_csr(rng, n_rows, ids, 40)
    mc = 3
    rp_h, cols_h, items_h = api._frequent_csr(rp, flat, n_rows, mc)
    got = api._coded_csr_device(rp, flat, n_rows, mc, torch.device("cuda"))
    assert got is not None and len(got.code_support) > 12_288
    assert np.array_equal(got.items, items_h)
    assert np.array_equal(got.support, np.bincount(cols_h, minlength=len(items_h)))
    assert np.array_equal(got.row_len, np.diff(rp_h))


def test_coded_input_declines_what_it_cannot_code(pkg):
    """Rows with a repeated or unsorted id, ids beyond the bitmap's span and UInt64 ids take the sorting path."""
    import torch

    api = import_module(pkg.__name__ + ".api")
    dev = torch.device("cuda")
    rp = np.array([0, 3, 5], np.int64)
    assert api._coded_csr_device(rp, np.array([1, 2, 2, 4, 7], np.int64), 2, 1, dev) is None  # repeated
    # A repeat across the boundary of two warp-wide steps of one row (entries 31 and 32).
    long_row = np.concatenate([np.arange(32), [31], np.arange(40, 50)]).astype(np.int64)
    assert api._coded_csr_device(np.array([0, len(long_row)], np.int64), long_row, 1, 1, dev) is None
    ok_row = np.concatenate([np.arange(32), np.arange(40, 50)]).astype(np.int64)
    assert api._coded_csr_device(np.array([0, len(ok_row)], np.int64), ok_row, 1, 1, dev) is not None
    assert api._coded_csr_device(rp, np.array([1, 3, 2, 4, 7], np.int64), 2, 1, dev) is None  # unsorted
    assert api._coded_csr_device(rp, np.array([1, 2, 3, 4, 1 << 27], np.int64), 2, 1, dev) is None  # span
    assert api._coded_csr_device(rp, np.array([1, 2, 3, 4, 7], np.uint64), 2, 1, dev) is None
    got = api._coded_csr_device(rp, np.array([1, 2, 3, 4, 7], np.int64), 2, 1, dev)
    assert got is not None and got.items.tolist() == [1, 2, 3, 4, 7]


def test_item_codes_report_an_id_outside_the_span(pkg):
    import torch

    lib = pkg.load_library()
    rp = torch.tensor([0, 2, 4], dtype=torch.int64, device="cuda")
    ids = torch.tensor([3, 9, 4, 40], dtype=torch.int64, device="cuda")
    span = 32
    bitmap = torch.empty(1, dtype=torch.int32, device="cuda")
    rank = torch.empty(2, dtype=torch.int64, device="cuda")
    codes = torch.empty(4, dtype=torch.int32, device="cuda")
    status = torch.empty(2, dtype=torch.int32, device="cuda")
    st = lib.etm_item_codes(rp.data_ptr(), ids.data_ptr(), 4, 2, 0, span, bitmap.data_ptr(), rank.data_ptr(),
                            codes.data_ptr(), status.data_ptr(), _stream())
    assert st == 0, lib.etm_last_error()
    assert status.cpu().tolist() == [1, 1]  # 40 lies outside [0, 32); its row is then not canonical either
    assert codes.cpu().tolist() == [0, 2, 1, -1]
    assert rank.cpu().tolist() == [0, 3]
    assert lib.etm_item_codes(rp.data_ptr(), ids.data_ptr(), 4, 2, 0, (1 << 26) + 1, bitmap.data_ptr(),
                              rank.data_ptr(), codes.data_ptr(), status.data_ptr(), _stream()) == 1
