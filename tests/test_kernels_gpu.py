"""Kernel-level GPU checks through the C ABI: each entry point against a host restatement."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import miner

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(pkg):
    return pkg.load_library()


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("n_rows,n_items,max_len", [(1, 37, 12), (63, 37, 12), (64, 37, 12), (65, 37, 12),
                                                    (1000, 37, 12), (100_003, 37, 12), (20_011, 3000, 90),
                                                    (3_001, 5000, 70)])
def test_build_bitvecs_is_byte_identical(pkg, lib, n_rows, n_items, max_len):
    """The shared-memory form (up to 3,072 columns; rows longer than a warp) and the global form, against the
    host restatement."""
    import torch

    rng = np.random.default_rng(n_rows + n_items)
    lens = rng.integers(0, max_len, n_rows)
    indptr = np.zeros(n_rows + 1, np.int64)
    np.cumsum(lens, out=indptr[1:])
    rows = [np.sort(rng.choice(n_items, size=l, replace=False)) for l in lens]
    ids = np.concatenate(rows).astype(np.int32) if rows else np.zeros(0, np.int32)
    want = miner.bitvecs_from_csr(indptr, ids, n_items, n_rows)
    ld = (n_rows + 63) // 64
    out = torch.full((n_items, ld), -1, dtype=torch.int64, device="cuda")
    d_ptr, d_ids = _dev(indptr), _dev(ids if len(ids) else np.zeros(1, np.int32))
    st = lib.etm_build_bitvecs(d_ptr.data_ptr(), d_ids.data_ptr(), len(ids), None, 0, n_rows, n_items, ld,
                               out.data_ptr(), _stream())
    assert st == 0, lib.etm_last_error()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)


def test_build_bitvecs_with_lut(pkg, lib):
    """ids go through an id -> column table; -1 and out-of-range ids are dropped (csr_to_bitvec.cu:46-73)."""
    import torch

    indptr = np.array([0, 3, 5, 6], np.int64)
    ids = np.array([7, 2, 9, 2, 100, 7], np.int32)
    lut = np.full(10, -1, np.int32)
    lut[2], lut[7] = 0, 1
    out = torch.zeros((2, 1), dtype=torch.int64, device="cuda")
    d = [_dev(indptr), _dev(ids), _dev(lut)]
    st = lib.etm_build_bitvecs(d[0].data_ptr(), d[1].data_ptr(), len(ids), d[2].data_ptr(), 10, 3, 2, 1,
                               out.data_ptr(), _stream())
    assert st == 0
    assert out.cpu().numpy().tolist() == [[0b011], [0b101]]


def test_popcount_and_gather(pkg, lib):
    import torch

    rng = np.random.default_rng(1)
    bv = rng.integers(0, 2**63, size=(50, 1001), dtype=np.int64).view(np.uint64)
    d = _dev(bv.view(np.int64))
    out = torch.empty(50, dtype=torch.int64, device="cuda")
    assert lib.etm_popcount_cols(d.data_ptr(), 50, 1000, 1001, out.data_ptr(), _stream()) == 0
    assert np.array_equal(out.cpu().numpy(), np.bitwise_count(bv[:, :1000]).sum(axis=1))
    cols = np.array([3, 0, 49], np.int32)
    g = torch.full((3, 1024), -1, dtype=torch.int64, device="cuda")
    d_cols = _dev(cols)
    assert lib.etm_gather_cols(d.data_ptr(), 1001, d_cols.data_ptr(), 3, 1000, g.data_ptr(), 1024, _stream()) == 0
    got = g.cpu().numpy().view(np.uint64)
    assert np.array_equal(got[:, :1000], bv[cols, :1000]) and not got[:, 1000:].any()


def test_synth_bernoulli_matches_host_twin(pkg, lib):
    import torch

    syn = pkg.synthetic
    thr = syn.bernoulli_thresholds(syn.dense_k2_probs(40, seed=4))
    n_rows = 3_000
    want = syn.bernoulli_bitvecs(thr, n_rows, seed=99)
    ld = (n_rows + 63) // 64
    out = torch.empty((40, ld), dtype=torch.int64, device="cuda")
    d_thr = _dev(thr.view(np.int64))
    assert lib.etm_synth_bernoulli(d_thr.data_ptr(), 40, n_rows, 99, out.data_ptr(), ld, _stream()) == 0
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)


def _host_groups(rows):
    n, w = rows.shape
    if n == 0:
        return []
    key = [tuple(r[: w - 1]) for r in rows]
    out, s = [], 0
    for t in range(1, n + 1):
        if t == n or key[t] != key[s]:
            if t - s >= 2:
                out.append((s, t - s))
            s = t
    return out


@pytest.mark.parametrize("width", [1, 2, 3])
def test_level_groups(pkg, lib, width):
    import torch

    rng = np.random.default_rng(width)
    rows = np.unique(rng.integers(0, 12, size=(400, width)), axis=0).astype(np.int32)
    rows = rows[np.all(np.diff(rows, axis=1) > 0, axis=1)] if width > 1 else rows
    n = len(rows)
    want = _host_groups(rows)
    gf = torch.empty(n, dtype=torch.int64, device="cuda")
    gs = torch.empty(n, dtype=torch.int32, device="cuda")
    co = torch.empty(n + 1, dtype=torch.int64, device="cuda")
    cnt = torch.empty(2, dtype=torch.int64, device="cuda")
    ws = torch.empty(3 + n // 4096 + 3, dtype=torch.int64, device="cuda")
    d_rows = _dev(rows)
    assert lib.etm_level_groups(d_rows.data_ptr(), n, width, gf.data_ptr(), gs.data_ptr(), co.data_ptr(),
                                cnt.data_ptr(), ws.data_ptr(), ws.numel(), _stream()) == 0, lib.etm_last_error()
    G, total = cnt.cpu().tolist()
    assert G == len(want)
    assert list(zip(gf[:G].cpu().tolist(), gs[:G].cpu().tolist())) == want
    pairs = [m * (m - 1) // 2 for _, m in want]
    assert co[: G + 1].cpu().tolist() == [0] + np.cumsum(pairs).tolist()
    assert total == sum(pairs)


def test_classify_labels(pkg, lib):
    """SKIP / INFER labels on the implication dataset against a brute-force host labelling."""
    import torch

    from tests.golden.make_golden import _implication

    rows_list = _implication()
    indptr = np.r_[0, np.cumsum([len(r) for r in rows_list])].astype(np.int64)
    items = np.concatenate([np.array(r) for r in rows_list]).astype(np.int64)
    n_rows = len(rows_list)
    res, col_items = miner.mine_transactions(indptr, items, n_rows, 0.01, 3, use_generator_pruning=True)
    l2_sets, l2_counts = res.levels[1]
    csr = miner.transaction_csr(indptr, items, n_rows, 0.01)
    bv = miner.bitvecs_from_csr(csr.indptr, csr.cols, csr.n_cols, n_rows)
    idx1 = miner.LevelIndex(res.levels[0][0], csr.n_cols)
    pos = miner.subset_positions(idx1, l2_sets)
    free2 = ~np.any(res.levels[0][1][pos] == l2_counts[:, None], axis=1)
    groups = _host_groups(l2_sets)
    cands, labels, inferred = [], [], []
    index = {tuple(r): t for t, r in enumerate(l2_sets.tolist())}
    for first, m in groups:
        for i in range(m):
            for j in range(i + 1, m):
                c = list(l2_sets[first + i]) + [l2_sets[first + j][1]]
                cands.append(c)
                subs = [tuple(x for x in c if x != y) for y in c]
                found = [index.get(s) for s in subs]
                if found[0] is None:
                    labels.append(1)
                    inferred.append(0)
                elif not all(free2[f] for f in found):
                    labels.append(2)
                    inferred.append(min(l2_counts[f] for f in found))
                else:
                    labels.append(0)
                    inferred.append(0)
    n = len(l2_sets)
    gf = torch.tensor([f for f, _ in groups], dtype=torch.int64, device="cuda")
    gs = torch.tensor([m for _, m in groups], dtype=torch.int32, device="cuda")
    co = torch.tensor([0] + np.cumsum([m * (m - 1) // 2 for _, m in groups]).tolist(), dtype=torch.int64, device="cuda")
    cls = torch.empty(len(cands), dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(len(cands), dtype=torch.int32, device="cuda")
    d = [_dev(l2_sets.astype(np.int32)), _dev(l2_counts.astype(np.int32)), _dev(free2.astype(np.uint8))]
    st = lib.etm_classify(d[0].data_ptr(), 2, n, d[1].data_ptr(), d[2].data_ptr(), gf.data_ptr(), gs.data_ptr(),
                          co.data_ptr(), 0, len(groups), 3, cls.data_ptr(), cnt.data_ptr(), _stream())
    assert st == 0
    got = cls.cpu().numpy()
    assert got.tolist() == labels
    inf = np.array(labels) == 2
    assert inf.any() and (np.array(labels) == 1).any()
    assert np.array_equal(cnt.cpu().numpy()[inf], np.array(inferred)[inf])
    # Inferred counts are exact: they equal the counted support.
    true = miner.count_itemsets(np.array(cands, dtype=np.int32)[inf], bv)
    assert np.array_equal(true, np.array(inferred)[inf])


@pytest.mark.parametrize("method", ["popcount"])
def test_pair_counts_all_pairs(pkg, method):
    """K=2 as one group: every pair count equals the host AND+popcount, word tails 1/31/32/33/65."""
    import torch

    from importlib import import_module

    eng = import_module(pkg.__name__ + ".engine").Engine(method=method)
    for n_words in (1, 31, 32, 33, 65):
        rng = np.random.default_rng(n_words)
        n_rows = n_words * 64 - 5
        n_f = 150
        bv = rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64).view(np.uint64)
        bv[:, -1] &= np.uint64((1 << 59) - 1)
        dev = torch.from_numpy(bv.view(np.int64)).cuda()
        fbv, ldp = eng.gather(dev.data_ptr(), n_words, np.arange(n_f), n_words)
        gen = import_module(pkg.__name__ + ".engine").Level(
            torch.arange(n_f, dtype=torch.int32, device="cuda")[:, None].contiguous(),
            torch.ones(n_f, dtype=torch.int32, device="cuda"))
        new, _ = eng.count_level(gen, fbv, ldp, n_words, 1, False, False)
        ii, jj = np.triu_indices(n_f, 1)
        want = np.bitwise_count(bv[ii] & bv[jj]).sum(axis=1)
        keep = want >= 1
        assert np.array_equal(new.rows.cpu().numpy(), np.stack([ii, jj], 1)[keep])
        assert np.array_equal(new.counts.cpu().numpy(), want[keep])
        del n_rows


def test_compaction_overflow_regrows(pkg):
    """A survivor count beyond the first output capacity regrows and repeats the chunk."""
    import torch

    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine(chunk_cands=1000)
    rng = np.random.default_rng(7)
    n_f, n_words = 700, 4
    bv = rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64)
    dev = torch.from_numpy(bv).cuda()
    fbv, ldp = eng.gather(dev.data_ptr(), n_words, np.arange(n_f), n_words)
    gen = engm.Level(torch.arange(n_f, dtype=torch.int32, device="cuda")[:, None].contiguous(),
                     torch.ones(n_f, dtype=torch.int32, device="cuda"))
    # Every pair survives at min_count 1 (random 256-bit columns always share a bit), far past the
    # first output capacity (65,536 rows), so the compaction regrows its output and repeats.
    new, stats = eng.count_level(gen, fbv, ldp, n_words, 1, False, False)
    ii, jj = np.triu_indices(n_f, 1)
    want = np.bitwise_count(bv.view(np.uint64)[ii] & bv.view(np.uint64)[jj]).sum(axis=1)
    assert new.n == len(ii) and stats.n_frequent == len(ii)
    assert np.array_equal(new.counts.cpu().numpy(), want)


@pytest.mark.parametrize("n_groups", [1, 5])
def test_bitmask_compaction_matches_dense_compaction(pkg, lib, n_groups):
    """etm_threshold_bits + etm_level_compact_bits give the rows, counts and order of etm_level_compact on the
    same dense counts and classes, for chunk sizes that end inside a 32-candidate word."""
    import torch

    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine()
    rng = np.random.default_rng(n_groups)
    # A width-2 level of n_groups prefix groups of uneven sizes: rows (p, s) lexsorted.
    sizes = rng.integers(2, 90, size=n_groups)
    rows = np.array([(p, s) for p, m in enumerate(sizes) for s in range(p + 1, p + 1 + m)], np.int32)
    gen = engm.Level(torch.from_numpy(rows).cuda(), torch.ones(len(rows), dtype=torch.int32, device="cuda"))
    G, total, grp_first, grp_size, cand_off = eng.groups(gen)
    assert G == n_groups and total == int((sizes * (sizes - 1) // 2).sum())
    counts = torch.from_numpy(rng.integers(0, 50, size=total).astype(np.int32)).cuda()
    cls = torch.from_numpy(rng.choice(np.array([0, 0, 1, 2], np.uint8), size=total)).cuda()
    s0 = torch.cuda.current_stream().cuda_stream
    outs = []
    for fused in (False, True):
        out_r = torch.full((total, 3), -1, dtype=torch.int32, device="cuda")
        out_c = torch.full((total,), -1, dtype=torch.int32, device="cuda")
        acc = torch.zeros(1, dtype=torch.int64, device="cuda")
        if fused:
            bits = torch.full(((total + 31) // 32 + 1,), -1, dtype=torch.int32, device="cuda")
            assert lib.etm_threshold_bits(counts.data_ptr(), cls.data_ptr(), total, 25, bits.data_ptr(), s0) == 0
            ws = torch.empty(engm.scan_words((total + 31) // 32), dtype=torch.int64, device="cuda")
            st = lib.etm_level_compact_bits(bits.data_ptr(), counts.data_ptr(), total, gen.rows.data_ptr(), 2,
                                            grp_first.data_ptr(), grp_size.data_ptr(), cand_off.data_ptr(), 0, G,
                                            out_r.data_ptr(), out_c.data_ptr(), total, acc.data_ptr(), ws.data_ptr(),
                                            ws.numel(), s0)
        else:
            ws = torch.empty(engm.scan_words(total), dtype=torch.int64, device="cuda")
            st = lib.etm_level_compact(counts.data_ptr(), cls.data_ptr(), total, gen.rows.data_ptr(), 2,
                                       grp_first.data_ptr(), grp_size.data_ptr(), cand_off.data_ptr(), 0, G, 25,
                                       out_r.data_ptr(), out_c.data_ptr(), total, acc.data_ptr(), ws.data_ptr(),
                                       ws.numel(), s0)
        assert st == 0, lib.etm_last_error()
        n = int(acc.item())
        outs.append((out_r[:n].cpu().numpy(), out_c[:n].cpu().numpy()))
    keep = (counts.cpu().numpy() >= 25) & (cls.cpu().numpy() != 1)
    assert len(outs[0][1]) == int(keep.sum()) > 0
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("max_len", [20, 700])
def test_pair_counts_rows_match_host(pkg, lib, max_len):
    """Row-wise K=2 (pairs_k2_rows.cu:54 restated): every pair count from the rows, through a column lut."""
    import torch

    rng = np.random.default_rng(max_len)
    n_rows, n_cols = 3000, 900
    lens = rng.integers(0, max_len, n_rows)
    lens[::97] = max_len  # some rows beyond the 512-entry shared slice when max_len is 700
    rows = [np.sort(rng.choice(n_cols, size=min(l, n_cols), replace=False)) for l in lens]
    indptr = np.zeros(n_rows + 1, np.int64)
    np.cumsum([len(r) for r in rows], out=indptr[1:])
    cols = np.concatenate(rows).astype(np.int32)
    keep = rng.random(n_cols) < 0.7  # columns that generate; the others map to -1
    gen = np.flatnonzero(keep)
    lut = np.full(n_cols, -1, np.int32)
    lut[gen] = np.arange(len(gen), dtype=np.int32)
    n_g = len(gen)
    want = np.zeros((n_g, n_g), np.int64)
    for r in rows:
        g = lut[r]
        g = g[g >= 0]
        ii, jj = np.triu_indices(len(g), 1)
        np.add.at(want, (g[ii], g[jj]), 1)
    want = want[np.triu_indices(n_g, 1)]
    out = torch.full((len(want),), -7, dtype=torch.int32, device="cuda")
    d = [_dev(indptr), _dev(cols), _dev(lut)]
    st = lib.etm_pair_counts_rows(d[0].data_ptr(), d[1].data_ptr(), len(cols), d[2].data_ptr(), n_cols, n_rows, n_g,
                                  out.data_ptr(), _stream())
    assert st == 0, lib.etm_last_error()
    assert np.array_equal(out.cpu().numpy(), want)


def _projection_reference(bits, ld, n_words, groups, stride):
    """Per group (prefix columns, member columns): each member's bits at the prefix rows, per segment of
    ETM_PROJ_SEG_WORDS words, every segment's piece padded to whole 4-word chunks, zeros to the stride."""
    seg = 1024
    out = []
    for (prefix, members), cl in zip(groups, stride):
        mask = np.ones(n_words * 64, bool)
        for c in prefix:
            mask &= bits[c]
        rows = []
        for m in members:
            words = []
            for s0 in range(0, n_words * 64, seg * 64):
                sel = bits[m][s0:s0 + seg * 64][mask[s0:s0 + seg * 64]]
                if len(sel):
                    pad = np.zeros((len(sel) + 255) // 256 * 256, np.uint8)
                    pad[:len(sel)] = sel
                    words.append(np.packbits(pad, bitorder="little").view(np.uint64))
            w = np.concatenate(words) if words else np.zeros(0, np.uint64)
            row = np.zeros(cl, np.uint64)
            row[:len(w)] = w
            rows.append(row)
        out.append(np.stack(rows))
    return out


@pytest.mark.parametrize("n_words,n_cols", [(1, 33), (3, 70), (64, 1000), (129, 4096)])
def test_rows_transpose_matches_host(lib, n_words, n_cols):
    """etm_rows_transpose: bit k of word c of row r is bit r of column 32 c + k (zero past n_cols)."""
    import torch

    rng = np.random.default_rng(n_words + n_cols)
    ld = max(32, (n_words + 31) // 32 * 32)
    fbv = rng.integers(0, 2**63, (n_cols, ld), dtype=np.int64)
    ldr = max(4, -(-(-(-n_cols // 32)) // 4) * 4)
    xt = torch.full((n_words * 64, ldr), -1, dtype=torch.int32, device="cuda")
    d = _dev(fbv)
    assert lib.etm_rows_transpose(d.data_ptr(), ld, n_words, n_cols, xt.data_ptr(), ldr, _stream()) == 0, \
        lib.etm_last_error()
    bits = np.unpackbits(fbv[:, :n_words].view(np.uint8), axis=1, bitorder="little")[:, :n_words * 64]
    padded = np.zeros((ldr * 32, n_words * 64), np.uint8)
    padded[:n_cols] = bits
    want = np.packbits(padded.T.reshape(n_words * 64, ldr, 32), axis=2, bitorder="little").reshape(
        n_words * 64, ldr * 4).view(np.uint32)
    assert np.array_equal(xt.cpu().numpy().view(np.uint32), want)


@pytest.mark.parametrize("form", ["cols", "rows"])
@pytest.mark.parametrize("blk", [0, 3, 240])
@pytest.mark.parametrize("n_words,width,n_cols", [(1, 2, 14), (1023, 2, 14), (1024, 3, 14), (1025, 2, 14),
                                                  (3001, 3, 14), (2500, 2, 14), (1100, 2, 300), (70, 3, 1000)])
def test_segmented_projection(pkg, lib, n_words, width, n_cols, blk, form):
    """etm_prefix_segments + the projection, column form (etm_project row-major, etm_project_blocked in blocks
    of blk members, chunk by chunk) or row form (etm_rows_transpose + etm_project_rows, either layout), against
    the host restatement: a dense prefix (more prefix rows in a segment than one pass lists), an empty prefix,
    the zero padding, and on wide column sets a group of every column (member ranks across chunks) beside
    groups of a few scattered columns (empty chunks skipped)."""
    import importlib

    import torch

    eng = importlib.import_module(pkg.__name__ + ".engine")
    rng = np.random.default_rng(n_words * 10 + width + n_cols)
    dens = np.array([0.9, 0.5, 0.06, 0.02, 0.0, 0.3] + [0.4] * (n_cols - 6))
    ld = max(32, (n_words + 31) // 32 * 32)
    bits = (rng.random((n_cols, n_words * 64)) < dens[:, None]).astype(np.uint8)
    words = np.packbits(bits, axis=1, bitorder="little").view(np.uint64)
    fbv_h = rng.integers(0, 2**63, (n_cols, ld), dtype=np.int64).view(np.uint64)  # garbage past n_words
    fbv_h[:, :n_words] = words
    plen = width - 1
    prefixes = [tuple(range(p, p + plen)) for p in (0, 1, 2, 3, 4)]
    groups = []
    level_rows = []
    for pre in prefixes:
        size = n_cols - plen - 4 if pre[0] == 1 and n_cols > 100 else int(rng.integers(1, 7))
        members = sorted(rng.choice(np.arange(plen + 4, n_cols), size=size, replace=False))
        groups.append((pre, members))
        for mbr in members:
            level_rows.append(list(pre) + [int(mbr)])
    rows = np.array(level_rows, np.int32)
    sizes = np.array([len(g[1]) for g in groups], np.int32)
    first = np.zeros(len(groups), np.int64)
    first[1:] = np.cumsum(sizes)[:-1]
    wg = np.array([4, 0, 2, 1, 3], np.int64)  # work entries in a different order than the groups
    cnt = []
    for g in wg:
        mask = np.ones(n_words * 64, bool)
        for c in groups[g][0]:
            mask &= bits[c].astype(bool)
        cnt.append(int(mask.sum()))
    cnt = np.array(cnt, np.int64)
    cl = eng.proj_stride(cnt, n_words)
    m = sizes[wg].astype(np.int64)
    m_rows = -(-m // blk) * blk if blk else m
    cb = np.zeros(len(wg) + 1, np.int64)
    np.cumsum(m_rows * cl, out=cb[1:])
    n_seg = -(-n_words // 1024)
    d_fbv, d_rows = _dev(fbv_h.view(np.int64)), _dev(rows)
    d_first, d_size, d_wg = _dev(first), _dev(sizes), _dev(wg)
    seg_off = torch.full((len(wg) * (n_seg + 1),), -7, dtype=torch.int64, device="cuda")
    out_words = torch.full((len(wg),), -7, dtype=torch.int64, device="cuda")
    st = lib.etm_prefix_segments(d_fbv.data_ptr(), ld, n_words, d_rows.data_ptr(), width, d_first.data_ptr(),
                                 d_wg.data_ptr(), len(wg), seg_off.data_ptr(), out_words.data_ptr(), None, 0,
                                 _stream())
    assert st == 0, lib.etm_last_error()
    cbuf = torch.full((int(cb[-1]),), -1, dtype=torch.int64, device="cuda")
    # Alternate the dynamic (work counter) and round-robin unit orders across the cases.
    ctr = torch.zeros(1, dtype=torch.int64, device="cuda")  # held for the call
    counter = ctr.data_ptr() if n_words % 2 else None
    d_cbase, d_cld = _dev(cb[:-1].copy()), _dev(cl)
    if form == "rows":
        ldr = max(4, -(-(-(-n_cols // 32)) // 4) * 4)
        xt = torch.empty((n_words * 64, ldr), dtype=torch.int32, device="cuda")
        st = lib.etm_rows_transpose(d_fbv.data_ptr(), ld, n_words, n_cols, xt.data_ptr(), ldr, _stream())
        assert st == 0, lib.etm_last_error()
        st = lib.etm_project_rows(d_fbv.data_ptr(), ld, n_words, xt.data_ptr(), ldr, d_rows.data_ptr(), width,
                                  d_first.data_ptr(), d_size.data_ptr(), d_wg.data_ptr(), len(wg),
                                  seg_off.data_ptr(), d_cbase.data_ptr(), d_cld.data_ptr(), blk, cbuf.data_ptr(),
                                  _stream())
    elif blk:
        st = lib.etm_project_blocked(d_fbv.data_ptr(), ld, n_words, d_rows.data_ptr(), width, d_first.data_ptr(),
                                     d_size.data_ptr(), d_wg.data_ptr(), len(wg), seg_off.data_ptr(),
                                     d_cbase.data_ptr(), d_cld.data_ptr(), blk, cbuf.data_ptr(), counter, _stream())
    else:
        st = lib.etm_project(d_fbv.data_ptr(), ld, n_words, d_rows.data_ptr(), width, d_first.data_ptr(),
                             d_size.data_ptr(), d_wg.data_ptr(), len(wg), seg_off.data_ptr(), d_cbase.data_ptr(),
                             d_cld.data_ptr(), cbuf.data_ptr(), counter, _stream())
    assert st == 0, lib.etm_last_error()
    got = cbuf.cpu().numpy().view(np.uint64)
    want = _projection_reference(bits.astype(bool), ld, n_words, [groups[g] for g in wg], cl)
    so = seg_off.cpu().numpy().reshape(len(wg), n_seg + 1)
    ow = out_words.cpu().numpy()
    for k in range(len(wg)):
        seg_counts = [int(((np.logical_and.reduce([bits[c].astype(bool) for c in groups[wg[k]][0]]))
                           [s * 65536:(s + 1) * 65536]).sum()) for s in range(n_seg)]
        expect_off = np.concatenate([[0], np.cumsum([((c + 63) // 64 + 3) // 4 * 4 for c in seg_counts])])
        assert np.array_equal(so[k], expect_off)
        assert ow[k] == expect_off[-1] <= cl[k]
        if blk:
            # Word w of member j at (j // blk) cl blk + (w // 4) 4 blk + (w // 2 % 2) 2 blk + (j % blk) 2 + w % 2.
            j = np.arange(m[k])[:, None]
            w = np.arange(cl[k])[None, :]
            idx = (j // blk) * cl[k] * blk + (w // 4) * 4 * blk + (w // 2 % 2) * 2 * blk + (j % blk) * 2 + w % 2
            block = got[cb[k]:cb[k + 1]][idx]
        else:
            block = got[cb[k]:cb[k + 1]].reshape(m[k], cl[k])
        assert np.array_equal(block, want[k]), f"work entry {k} (group {wg[k]})"


@pytest.mark.parametrize("long_rows", [False, True])
def test_triple_counts_rows_match_host(pkg, lib, long_rows):
    """Row-wise K=3 (k3_rows.cu:50-140 restated on the prefix-group layout): the counts of a candidate range
    from the rows, only for candidates classed as counted; the other classes keep their values."""
    import torch

    rng = np.random.default_rng(7 + long_rows)
    n_rows, n_cols = 2500, 700 if long_rows else 120
    lens = rng.integers(0, 14, n_rows)
    if long_rows:
        lens[::211] = 600  # beyond the 512-entry shared slice
    rows = [np.sort(rng.choice(n_cols, size=min(l, n_cols), replace=False)) for l in lens]
    indptr = np.zeros(n_rows + 1, np.int64)
    np.cumsum([len(r) for r in rows], out=indptr[1:])
    cols = np.concatenate(rows).astype(np.int32)
    gen = np.flatnonzero(rng.random(n_cols) < 0.8)  # columns that generate
    lut = np.full(n_cols, -1, np.int32)
    lut[gen] = np.arange(len(gen), dtype=np.int32)
    ng = len(gen)
    # A K=2 generating level: a random set of pairs (u < v) of generator indices, lexsorted.
    iu, iv = np.triu_indices(ng, 1)
    keep = rng.random(len(iu)) < (0.05 if long_rows else 0.3)
    pairs = np.stack([iu[keep], iv[keep]], 1).astype(np.int32)
    us, starts, counts = np.unique(pairs[:, 0], return_index=True, return_counts=True)
    sel = counts >= 2
    us, starts, counts = us[sel], starts[sel], counts[sel]
    G = len(us)
    cand = counts.astype(np.int64) * (counts - 1) // 2
    cand_off = np.zeros(G + 1, np.int64)
    np.cumsum(cand, out=cand_off[1:])
    grp_of = np.full(ng, -1, np.int32)
    grp_of[us] = np.arange(G, dtype=np.int32)
    total = int(cand_off[-1])
    want = np.zeros(total, np.int64)
    for r in rows:
        g = lut[r]
        g = g[g >= 0]
        for a, u in enumerate(g):
            k = grp_of[u]
            if k < 0:
                continue
            mem = pairs[starts[k]:starts[k] + counts[k], 1]
            idx = np.searchsorted(mem, g[a + 1:])
            ok = (idx < len(mem)) & (mem[np.minimum(idx, len(mem) - 1)] == g[a + 1:])
            idx = idx[ok]
            ii, jj = np.triu_indices(len(idx), 1)
            m = counts[k]
            t = cand_off[k] + idx[ii] * (2 * m - idx[ii] - 1) // 2 + (idx[jj] - idx[ii] - 1)
            np.add.at(want, t, 1)
    base, n_c = total // 5, total - total // 5 - 3
    cls = rng.integers(0, 3, n_c).astype(np.uint8)  # 0 counted; other classes keep their values
    expect = np.where(cls == 0, want[base:base + n_c], -7)
    out = torch.full((n_c,), -7, dtype=torch.int32, device="cuda")
    d = [_dev(indptr), _dev(cols), _dev(lut), _dev(pairs), _dev(grp_of), _dev(starts.astype(np.int64)),
         _dev(counts.astype(np.int32)), _dev(cand_off), _dev(cls)]
    st = lib.etm_triple_counts_rows(d[0].data_ptr(), d[1].data_ptr(), len(cols), d[2].data_ptr(), n_cols, n_rows,
                                    d[3].data_ptr(), d[4].data_ptr(), ng, d[5].data_ptr(), d[6].data_ptr(),
                                    d[7].data_ptr(), base, n_c, d[8].data_ptr(), out.data_ptr(), _stream())
    assert st == 0, lib.etm_last_error()
    assert np.array_equal(out.cpu().numpy(), expect)


@pytest.mark.parametrize("n_split", [1, 7, 94])
def test_split_tiles_add_up_to_the_whole_counts(pkg, lib, n_split):
    """etm_count_tiles_split: the word range of every tile-pair cut into n_split parts whose partial counts
    are added atomically gives the counts of etm_count_tiles, including word tails and a prefix AND."""
    import torch

    from importlib import import_module

    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine(method="popcount")
    rng = np.random.default_rng(n_split)
    n_f, n_words = 150, 2999
    bv = rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64)
    bv &= rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64)
    dev = torch.from_numpy(bv).cuda()
    fbv, ldp = eng.gather(dev.data_ptr(), n_words, np.arange(n_f), n_words)
    # Width 2: prefix column 0 with members 1..149 (one group, the prefix ANDed in per word).
    rows = np.stack([np.zeros(n_f - 1, np.int32), np.arange(1, n_f, dtype=np.int32)], axis=1)
    gen = engm.Level(torch.from_numpy(rows).cuda(), torch.ones(n_f - 1, dtype=torch.int32, device="cuda"))
    G, total, gf, gs, co = eng.groups(gen)
    m = n_f - 1
    nt = (m + 63) // 64
    wg, wo = eng._work(np.zeros(1, np.int64), np.array([nt * (nt + 1) // 2]))
    st = torch.cuda.current_stream().cuda_stream
    want = torch.full((total,), -5, dtype=torch.int32, device="cuda")
    assert lib.etm_count_tiles(fbv.data_ptr(), ldp, n_words, gen.rows.data_ptr(), 2, gf.data_ptr(), gs.data_ptr(),
                               co.data_ptr(), wg.data_ptr(), wo.data_ptr(), 1, 0, None, 0, want.data_ptr(), st) == 0
    got = torch.zeros(total, dtype=torch.int32, device="cuda")
    assert lib.etm_count_tiles_split(fbv.data_ptr(), ldp, n_words, gen.rows.data_ptr(), 2, gf.data_ptr(),
                                     gs.data_ptr(), co.data_ptr(), wg.data_ptr(), wo.data_ptr(), 1,
                                     nt * (nt + 1) // 2, 0, None, n_split, got.data_ptr(), st) == 0, \
        lib.etm_last_error()
    w = want.cpu().numpy()
    assert (w >= 0).all()
    assert np.array_equal(got.cpu().numpy(), w)
    ii, jj = np.triu_indices(m, 1)
    host = np.bitwise_count(bv.view(np.uint64)[0] & bv.view(np.uint64)[1 + ii] & bv.view(np.uint64)[1 + jj]).sum(1)
    assert np.array_equal(w, host)
