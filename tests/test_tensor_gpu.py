"""The tcgen05 Gram path: bit-exact against the popcount path and the golden results.

Counts are integers; the tensor-core path accumulates 0/1 products in f32,
which is exact while a group holds at most 2^24 rows. The tolerance is zero.
"""

from __future__ import annotations

import json
from importlib import import_module
from pathlib import Path

import numpy as np
import pytest

from tests.conftest import case_input
from tests.helpers import digest_pairs, table_of

pytestmark = pytest.mark.gpu

CASES = [c["name"] for c in json.loads((Path(__file__).parent / "golden" / "cases.json").read_text())["cases"]]


def _k2(pkg, bv_np, method, elem=2):
    import torch

    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine(method=method, tc_elem=elem, small_group=1)
    n_f, n_words = bv_np.shape
    dev = torch.from_numpy(np.ascontiguousarray(bv_np).view(np.int64)).cuda()
    fbv, ldp = eng.gather(dev.data_ptr(), n_words, np.arange(n_f), n_words)
    gen = engm.Level(torch.arange(n_f, dtype=torch.int32, device="cuda")[:, None].contiguous(),
                     torch.ones(n_f, dtype=torch.int32, device="cuda"))
    new, _ = eng.count_level(gen, fbv, ldp, n_words, 1, False, False, n_words * 64)
    assert eng.used_tensor == (method == "tensor")
    return new.rows.cpu().numpy(), new.counts.cpu().numpy()


# Element codes: 1 e4m3, 2 f16 (blocks of 256 members), 4 packed e2m1 (blocks of 240); + 16 is accepted and ignored.
ELEMS = [1, 2, 4, 1 | 16]


@pytest.mark.parametrize("elem", ELEMS)
@pytest.mark.parametrize("n_f,n_words", [(2, 1), (127, 31), (128, 32), (129, 33), (239, 7), (240, 9), (241, 2),
                                         (255, 4), (256, 5), (257, 3), (300, 65), (481, 3), (513, 6)])
def test_pair_counts_match_popcount(pkg, n_f, n_words, elem):
    rng = np.random.default_rng(n_f * 1000 + n_words)
    bv = rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64).view(np.uint64)
    bv &= rng.integers(0, 2**63, size=(n_f, n_words), dtype=np.int64).view(np.uint64)  # density 1/4
    want_rows, want = _k2(pkg, bv, "popcount")
    got_rows, got = _k2(pkg, bv, "tensor", elem)
    assert np.array_equal(got_rows, want_rows)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("elem", [1, 2, 4])
def test_counts_exact_up_to_2_24_rows(pkg, elem):
    """All-ones columns over 2^24 - 64 rows: every pair count equals the row count exactly."""
    n_rows = (1 << 24) - 64
    n_words = n_rows // 64
    n_f = 130
    bv = np.full((n_f, n_words), np.uint64(0xFFFFFFFFFFFFFFFF), dtype=np.uint64)
    bv[5, 7] = np.uint64(0)  # one column 64 short: its pairs count n_rows - 64
    rows, counts = _k2(pkg, bv, "tensor", elem)
    want = np.full(len(rows), n_rows, dtype=np.int64)
    want[(rows[:, 0] == 5) | (rows[:, 1] == 5)] = n_rows - 64
    assert len(rows) == n_f * (n_f - 1) // 2
    assert np.array_equal(counts, want)


@pytest.mark.parametrize("elem", [1, 2, 4])
@pytest.mark.parametrize("name", ["implication_plain", "implication_infer", "implication_prune", "plain_small_plain",
                                  "dense_k2_small", "deep_sparse_small", "word_tail_2049", "word_tail_65"])
def test_tensor_engine_matches_golden(pkg, golden_cases, name, elem):
    case = golden_cases[name]
    indptr, items, n_rows = case_input(pkg, case)
    engm = import_module(pkg.__name__ + ".engine")
    eng = engm.Engine(method="tensor", tc_elem=elem, small_group=4)
    got = pkg.apriori(table_of(indptr, items, n_rows), min_support=case["min_support"], max_length=case["max_length"],
                      use_gpu=True, prune_equal_support=case["prune_equal_support"],
                      use_generator_pruning=case["use_generator_pruning"], engine=eng, warn_complexity=False)
    assert digest_pairs(pkg.result_pairs(got, n_rows)) == case["digest"]


@pytest.mark.parametrize("elem", [1, 4])
def test_random_bits_exact_near_2_24_rows(pkg, elem):
    """Random bits of density 1/2 over 2^24 - 64 rows: pair counts near 2^22 with arbitrary low bits, the
    tensor path equal to the popcount path (f32 accumulation stays exact below 2^24)."""
    n_rows = (1 << 24) - 64
    n_words = n_rows // 64
    n_f = 250  # two blocks of either size: diagonal and off-diagonal block pairs
    rng = np.random.default_rng(24)
    bv = rng.integers(-(2**63), 2**63 - 1, size=(n_f, n_words), dtype=np.int64, endpoint=True).view(np.uint64)
    want_rows, want = _k2(pkg, bv, "popcount")
    got_rows, got = _k2(pkg, bv, "tensor", elem)
    assert np.array_equal(got_rows, want_rows)
    assert np.array_equal(got, want)
    assert (want & 1).any() and (want % 1024 != 0).any() and want.max() > (1 << 21)


def test_dense_bernoulli_tensor_matches_popcount(pkg):
    """A dense workload (several 128-member tiles per group) mined both ways."""
    import torch

    syn = pkg.synthetic
    engm = import_module(pkg.__name__ + ".engine")
    p = np.minimum(syn.dense_k2_probs(400, seed=9) * 3, 0.9)
    bv = syn.bernoulli_bitvecs(syn.bernoulli_thresholds(p), 20_000, seed=5)
    dev = torch.from_numpy(bv.view(np.int64)).cuda().view(torch.uint64)
    a = engm.Engine(method="popcount").mine(dev, 20_000, 0.01, 3).host_levels()
    b = engm.Engine(method="tensor").mine(dev, 20_000, 0.01, 3).host_levels()
    assert len(a) == len(b)
    for (ra, ca), (rb, cb) in zip(a, b):
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb)


def _gram_groups(lib, elem, seed=11, blocked=False):
    """Member words of several groups of different sizes and lengths on the device, laid out as the
    projection lays them out (row-major, or blocked in blocks of the kernel's block size), with their host
    Gram (upper triangles, candidate order) and work lists."""
    import torch

    t = lib.etm_gram_block_members(elem)
    rng = np.random.default_rng(seed)
    sizes = np.array([300, 1, 2, 257, 513, 40, 481], np.int64)
    cw = np.array([64, 2, 3, 130, 17, 1, 5], np.int64)  # words per member row (odd counts end in a part stage)
    cld = (cw + 31) // 32 * 32
    rows_alloc = -(-sizes // t) * t if blocked else sizes
    cbase = np.zeros(len(sizes), np.int64)
    cbase[1:] = np.cumsum(rows_alloc * cld)[:-1]
    buf = np.zeros(int((rows_alloc * cld).sum()), np.uint64)
    want = []
    for g in range(len(sizes)):
        m, w = int(sizes[g]), int(cw[g])
        x = rng.integers(0, 2**63, size=(m, w), dtype=np.int64).view(np.uint64)
        x &= rng.integers(0, 2**63, size=(m, w), dtype=np.int64).view(np.uint64)
        if blocked:
            j = np.arange(m)[:, None]
            ww = np.arange(w)[None, :]
            buf[cbase[g] + (j // t) * cld[g] * t + (ww // 4) * 4 * t + (ww // 2 % 2) * 2 * t + (j % t) * 2 + ww % 2] = x
        else:
            buf[cbase[g]:cbase[g] + m * cld[g]].reshape(m, cld[g])[:, :w] = x
        bits = np.unpackbits(x.view(np.uint8), axis=1).astype(np.int64)
        want.append((bits @ bits.T)[np.triu_indices(m, 1)])
    want = np.concatenate(want).astype(np.int32)
    cand_off = np.zeros(len(sizes) + 1, np.int64)
    np.cumsum(sizes * (sizes - 1) // 2, out=cand_off[1:])
    nb = (sizes + t - 1) // t
    work_off = np.zeros(len(sizes) + 1, np.int64)
    np.cumsum(nb * (nb + 1) // 2, out=work_off[1:])
    d = {k: torch.from_numpy(v).cuda() for k, v in dict(
        buf=buf.view(np.int64), cbase=cbase, cwords=cw, cld=cld, size=sizes.astype(np.int32),
        cand_off=cand_off, wg=np.arange(len(sizes), dtype=np.int64), wo=work_off).items()}
    return t, d, want, len(sizes), int(work_off[-1])


def _gram_args(d):
    return (d["buf"].data_ptr(), d["cbase"].data_ptr(), d["cwords"].data_ptr(), d["cld"].data_ptr(),
            d["size"].data_ptr(), d["cand_off"].data_ptr(), d["wg"].data_ptr(), d["wo"].data_ptr())


@pytest.mark.parametrize("blocked", [False, True])
@pytest.mark.parametrize("elem", [1 | 16, 2, 4])
@pytest.mark.parametrize("with_counter", [True, False])
def test_wide_kernel_claimed_and_round_robin_items_agree(pkg, with_counter, elem, blocked):
    """etm_count_tiles_tc over several groups of different sizes and lengths, row-major or blocked member
    rows: block pairs claimed from a work counter or taken round-robin give the same counts, equal to a host
    Gram."""
    import torch

    lib = pkg.load_library()
    t, d, want, n_work, n_items = _gram_groups(lib, elem, blocked=blocked)
    assert t == (240 if elem == 4 else 256)
    out = torch.full((len(want),), -7, dtype=torch.int32, device="cuda")
    counter = torch.full((1,), 12345, dtype=torch.int64, device="cuda")  # zeroed by the call
    code = elem | (32 if blocked else 0)
    st = lib.etm_count_tiles_tc(*_gram_args(d), n_work, n_items, 0, None, code, out.data_ptr(),
                                counter.data_ptr() if with_counter else None, torch.cuda.current_stream().cuda_stream)
    assert st == 0, lib.etm_last_error()
    assert np.array_equal(out.cpu().numpy(), want)
    if with_counter:
        # Each CTA starts on item blockIdx.x, claims one item after each it finishes, and stops at its
        # first claim past the end: (items - grid) claims that succeed + grid that fail = items.
        assert int(counter.item()) == n_items


@pytest.mark.parametrize("elem", [1, 4])
def test_gram_fused_threshold(pkg, elem):
    """etm_count_tiles_tc_sel: the survivor bitmask holds exactly the counted candidates reaching min_count,
    their counts are written, every other slot is left untouched; SKIP and INFER classes are not counted."""
    import torch

    lib = pkg.load_library()
    _, d, want, n_work, n_items = _gram_groups(lib, elem, seed=5)
    n = len(want)
    rng = np.random.default_rng(3)
    cls = rng.choice(np.array([0, 0, 0, 1, 2], np.uint8), size=n)
    mc = int(np.median(want[want > 0]))
    cls_d = torch.from_numpy(cls).cuda()
    out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    bits = torch.zeros(((n + 31) // 32 + 1,), dtype=torch.int32, device="cuda")
    st = lib.etm_count_tiles_tc_sel(*_gram_args(d), n_work, n_items, 0, cls_d.data_ptr(), elem, mc, out.data_ptr(),
                                    bits.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert st == 0, lib.etm_last_error()
    surv = (cls == 0) & (want >= mc)
    got_bits = np.unpackbits(bits.cpu().numpy().view(np.uint8), bitorder="little")
    assert np.array_equal(got_bits[:n].astype(bool), surv)
    assert not got_bits[n:].any()
    o = out.cpu().numpy()
    assert np.array_equal(o[surv], want[surv])
    assert (o[~surv] == -7).all()


def test_bounded_wait_give_up_reports_timeout_and_device_stays_usable(pkg):
    """The Gram's and the column-form projection's first waits set to give up at once: each kernel abandons its
    work, drains what it issued, and the status word reads ETM_ETIMEOUT; then, with the default limits, the
    same mine on the same device is exact again. (The row-major projection has no device waits.)"""
    import torch

    lib = pkg.load_library()
    engm = import_module(pkg.__name__ + ".engine")
    syn = pkg.synthetic
    p = np.minimum(syn.dense_k2_probs(300, seed=9) * 3, 0.9)
    bv = syn.bernoulli_bitvecs(syn.bernoulli_thresholds(p), 20_000, seed=5)
    dev = torch.from_numpy(bv.view(np.int64)).cuda().view(torch.uint64)
    want = engm.Engine(method="popcount").mine(dev, 20_000, 0.01, 3).host_levels()
    assert lib.etm_device_status(None) == 0
    try:
        for gram_ns, proj_ns in ((0, -1), (-1, 0)):
            assert lib.etm_set_wait_limits(gram_ns, proj_ns) == 0
            with pytest.raises(RuntimeError, match="bounded wait"):
                engm.Engine(method="tensor", proj_rows=False).mine(dev, 20_000, 0.01, 3)
            assert lib.etm_device_status(None) == 0  # read and cleared by the engine
    finally:
        lib.etm_set_wait_limits(-1, -1)
    got = engm.Engine(method="tensor").mine(dev, 20_000, 0.01, 3).host_levels()
    assert len(got) == len(want)
    for (ra, ca), (rb, cb) in zip(want, got):
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb)
