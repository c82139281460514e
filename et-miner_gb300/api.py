"""``apriori()``: the drop-in for ET-Miner's GPU route (core/apriori.py:303-754).

Same signature, parameter validation and error types as the reference's
``apriori``. Two inputs reach the GB300 engine:

* ``bitvecs=(array, col_to_item, n_transactions)``: the caller's
  C-contiguous uint64 device array ``(n_cols, ceil(N/64))`` (any object with
  ``__cuda_array_interface__``, or a torch CUDA tensor), read only
  (core/apriori.py:477-548);
* ``transactions`` with ``use_gpu=True``: a list column (polars DataFrame or
  LazyFrame when polars is installed, a pyarrow Table, a dict of lists, or a
  plain list of item lists). On the device the items are deduplicated per
  row and counted, the frequent ones coded to columns in ascending id order,
  and the column bitvectors built by ``etm_build_bitvecs`` (the reference's
  input layer, gpu/input_layer.py:469-544 and gpu/csr_bitvec.py:63-155).

The routes this engine does not implement (the CPU route, SON streaming,
several GPUs, the per-level parquet flush, resume, anchors) raise
``ValueError`` naming the option, rather than silently answering another
question (the reference's own rule, core/apriori.py:109-251).

The result is a polars DataFrame when polars is importable, else a pyarrow
Table, with columns ``itemset`` (list of ascending item ids: Int64, or the
input's UInt64 / wide dtype kept, core/result.py:30-54) and ``support``
(Float64 = count / N). Row order is not part of the contract.
"""

from __future__ import annotations

import math
import numbers
import os
import time
import warnings
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from math import comb
from typing import Any

import numpy as np

from . import flush as _flush
from .engine import Engine, MineOutput, min_count

try:  # optional: results come back as polars frames when it is installed
    import polars as _pl
except Exception:  # pragma: no cover - polars is absent in the build image
    _pl = None

try:  # optional: pyarrow tables in and out when it is installed
    import pyarrow as pa
except Exception:  # pragma: no cover - the GPU machine has no pyarrow
    pa = None


@dataclass
class Phase:
    name: str
    ms: float
    extra: dict = field(default_factory=dict)


class ProfilingSession:
    """Per-phase wall times of one mining call (the reference's core/profiling.py:26-177, in brief).

    ``phases`` holds one entry per level (``k1``, ``k2``, ...) with the
    candidates, frequent itemsets, prefix groups and launches of the level.
    """

    def __init__(self) -> None:
        self.phases: list[Phase] = []
        self._open: tuple[str, float] | None = None

    def start_phase(self, name: str) -> None:
        self._open = (name, time.perf_counter())

    def end_phase(self, **extra) -> None:
        if self._open is not None:
            name, t0 = self._open
            self.phases.append(Phase(name, (time.perf_counter() - t0) * 1e3, dict(extra)))
            self._open = None

    def record_phase(self, name: str, ms: float, **extra) -> None:
        self.phases.append(Phase(name, ms, dict(extra)))

    @property
    def total_ms(self) -> float:
        return sum(p.ms for p in self.phases)

    def summary(self) -> str:
        return "\n".join(f"{p.name:>6s} {p.ms:10.2f} ms {p.extra}" for p in self.phases)


def _warn_complexity(n_frequent_items: int, min_support: float) -> None:
    """Warn when the pair count is large (core/apriori.py:38-61)."""
    n_pairs = comb(n_frequent_items, 2) if n_frequent_items > 1 else 0
    if n_pairs > 10_000_000:
        warnings.warn(f"Very large computation ahead: {n_frequent_items:,} frequent items, {n_pairs:,} candidate "
                      f"pairs (min_support={min_support})", UserWarning, stacklevel=3)
    elif n_pairs > 1_000_000:
        warnings.warn(f"Large computation: {n_pairs:,} candidate pairs.", UserWarning, stacklevel=3)


def _validate_parameters(min_support, max_length, batch_size, sparse_from_k=None, prune_apriori=True) -> None:
    """Parameter checks of core/apriori.py:64-106."""
    if isinstance(min_support, bool) or not isinstance(min_support, (int, float)):
        raise TypeError(f"min_support must be numeric, got {type(min_support).__name__}")
    if not 0.0 <= min_support <= 1.0:
        raise ValueError(f"min_support must be in range [0.0, 1.0], got {min_support}")
    if max_length is not None:
        if isinstance(max_length, bool) or not isinstance(max_length, int):
            raise TypeError(f"max_length must be int or None, got {type(max_length).__name__}")
        if max_length < 1:
            raise ValueError(f"max_length must be >= 1, got {max_length}")
    if batch_size is not None:
        if isinstance(batch_size, bool) or not isinstance(batch_size, int):
            raise TypeError(f"batch_size must be int or None, got {type(batch_size).__name__}")
        if batch_size < 1:
            raise ValueError(f"batch_size must be >= 1, got {batch_size}")
    if sparse_from_k is not None:
        raise ValueError("sparse_from_k was removed: the miner keeps dense bitvectors at every level. Drop the argument.")
    if not isinstance(prune_apriori, bool):
        raise TypeError(f"prune_apriori must be bool, got {type(prune_apriori).__name__}")
    if not prune_apriori:
        raise ValueError("prune_apriori=False was removed: every candidate's (k-1)-subsets are tested. Drop the argument.")


def _unsupported(**opts) -> None:
    """Reject the routes and options outside this engine's path (one GPU, counting path only)."""
    for name, (value, why) in opts.items():
        if value:
            raise ValueError(f"{name} is not supported by the GB300 counting engine: {why}")


# ---- input: transactions -> CSR of frequent columns ------------------------------

def _coded(flat: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(int64 rank of every item among the distinct items, those items sorted): the coding of non-integer
    item ids (``_coded_items``, core/apriori.py:277-284). Ranks follow the item order, so ascending codes
    are ascending items; results map back through the sorted items."""
    labels, codes = np.unique(flat, return_inverse=True)
    return codes.astype(np.int64).ravel(), labels


def _label_values(flat: np.ndarray) -> np.ndarray:
    """Non-integer items as a result emits them (``_emitted_items``, core/result.py:82-92): floats as
    float64, anything else (strings, categorical values) as strings."""
    if np.issubdtype(flat.dtype, np.floating):
        return flat.astype(np.float64)
    return flat.astype(str)


def _list_column(transactions, item_col: str):
    """(indptr int64, flat item values, their numpy dtype, labels) of a transaction list column.

    Accepts a polars DataFrame/LazyFrame or pyarrow Table (when installed), a
    CSR object with ``indptr`` and ``items`` arrays, a dict ``{item_col: rows}``
    or a list of item lists. Null lists are rows without items; null entries
    are no items. Integer ids come back as they are with ``labels`` None;
    strings, floats and categorical values come back coded (int64 ranks) with
    ``labels`` the sorted distinct values the ranks stand for.
    """
    if hasattr(transactions, "indptr") and hasattr(transactions, "items") and not isinstance(transactions, dict):
        indptr = np.asarray(transactions.indptr, dtype=np.int64)
        flat = np.asarray(transactions.items)
        if np.issubdtype(flat.dtype, np.integer):
            return indptr, flat, flat.dtype, None
        codes, labels = _coded(_label_values(flat))
        return indptr, codes, codes.dtype, labels
    if isinstance(transactions, dict):
        return _python_rows(transactions[item_col])
    if isinstance(transactions, (list, tuple)):
        return _python_rows(transactions)
    arr = None
    if _pl is not None and isinstance(transactions, (_pl.DataFrame, _pl.LazyFrame)):
        lf = transactions.lazy() if isinstance(transactions, _pl.DataFrame) else transactions
        arr = lf.select(_pl.col(item_col)).collect().get_column(item_col).to_arrow()
    elif pa is not None and isinstance(transactions, pa.Table):
        arr = transactions.column(item_col)
    if arr is None:
        raise TypeError(f"transactions must be a DataFrame, pyarrow Table, CSR, dict or list of lists, "
                        f"got {type(transactions).__name__}")
    if isinstance(arr, pa.ChunkedArray):
        arr = arr.combine_chunks()
    if not (pa.types.is_list(arr.type) or pa.types.is_large_list(arr.type)):
        raise TypeError(f"column {item_col!r} must be a list column, got {arr.type}")
    vt = arr.type.value_type
    if not (pa.types.is_integer(vt) or pa.types.is_floating(vt) or pa.types.is_string(vt)
            or pa.types.is_large_string(vt) or pa.types.is_dictionary(vt)):
        raise TypeError(f"items must be integers, floats, strings or categorical values, got {vt}")
    offsets = np.asarray(arr.offsets.to_numpy(zero_copy_only=False), dtype=np.int64)
    n = len(arr)
    vals = arr.values.slice(offsets[0], offsets[-1] - offsets[0])
    valid = np.ones(len(vals), dtype=bool)
    if vals.null_count:
        valid &= ~np.asarray(vals.is_null().to_numpy(zero_copy_only=False))
    if arr.null_count:
        valid &= np.repeat(~np.asarray(arr.is_null().to_numpy(zero_copy_only=False)), np.diff(offsets))
    if pa.types.is_dictionary(vt):
        vals = vals.cast(vt.value_type)  # categorical values are emitted as their strings
    if pa.types.is_integer(vt):
        flat = np.asarray(vals.fill_null(0).to_numpy(zero_copy_only=False))
    else:
        flat = np.asarray(vals.to_numpy(zero_copy_only=False))
    rid = np.repeat(np.arange(n, dtype=np.int64), np.diff(offsets))[valid]
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rid, minlength=n), out=indptr[1:])
    flat = flat[valid]
    if pa.types.is_integer(vt):
        return indptr, flat, flat.dtype, None
    codes, labels = _coded(_label_values(flat))
    return indptr, codes, codes.dtype, labels


def _python_rows(rows):
    rows = [[] if r is None else [x for x in r if x is not None] for r in rows]
    indptr = np.zeros(len(rows) + 1, dtype=np.int64)
    np.cumsum([len(r) for r in rows], out=indptr[1:])
    flat_list = [x for r in rows for x in r]
    if all(isinstance(x, numbers.Integral) and not isinstance(x, bool) for x in flat_list):
        big = any(x > np.iinfo(np.int64).max for x in flat_list)
        flat = np.array(flat_list, dtype=np.uint64 if big else np.int64)
        return indptr, flat, flat.dtype, None
    kinds = {type(x) for x in flat_list}
    if all(issubclass(t, numbers.Real) and not issubclass(t, bool) for t in kinds):
        flat = np.array(flat_list, dtype=np.float64)
    elif all(issubclass(t, str) for t in kinds):
        flat = np.array(flat_list, dtype=str)
    else:
        raise TypeError(f"items must all be integers, all numbers or all strings, got {sorted(t.__name__ for t in kinds)}")
    codes, labels = _coded(_label_values(flat))
    return indptr, codes, codes.dtype, labels


def _frequent_csr(indptr: np.ndarray, flat: np.ndarray, n_rows: int, mc: int):
    """(row_ptr, column ids int32, items of the columns): rows deduplicated, columns = items with count >= mc.

    The host restatement of ``_frequent_csr_device`` (the tests check one against the other)."""
    rid = np.repeat(np.arange(n_rows, dtype=np.int64), np.diff(indptr))
    items, inv = np.unique(flat, return_inverse=True)
    key = rid * max(1, len(items)) + inv
    key = np.unique(key)
    rid = key // max(1, len(items))
    inv = key % max(1, len(items))
    counts = np.bincount(inv, minlength=len(items))
    keep = counts >= max(1, mc)
    remap = np.cumsum(keep) - 1
    sel = keep[inv]
    cols = remap[inv[sel]].astype(np.int32)
    rid = rid[sel]
    row_ptr = np.zeros(n_rows + 1, dtype=np.int64)
    np.cumsum(np.bincount(rid, minlength=n_rows), out=row_ptr[1:])
    return row_ptr, cols, items[keep]


def _frequent_csr_device(indptr: np.ndarray, flat: np.ndarray, n_rows: int, mc: int, device):
    """``_frequent_csr`` on the device: (row_ptr int64 [n_rows+1] and column ids int32 as device tensors, the
    items of the columns, the rows' lengths and the columns' supports on the host).

    The same steps as the host version (sort the ids, drop repeated (row, item) pairs, keep the items
    with count >= mc, number them in ascending id order), with device sorts; UInt64 ids are sorted
    through their sign-flipped int64 bits, which orders them as unsigned values.
    """
    import torch

    sign = -(2**63)
    wide = flat.dtype == np.uint64
    host = np.ascontiguousarray(flat).view(np.int64) if wide else np.ascontiguousarray(flat).astype(np.int64, copy=False)
    vals = torch.from_numpy(host).to(device)
    if wide:
        vals = vals ^ sign
    lens = torch.from_numpy(np.diff(indptr).astype(np.int64)).to(device)
    rid = torch.repeat_interleave(torch.arange(n_rows, dtype=torch.int64, device=device), lens)
    items, inv = torch.unique(vals, sorted=True, return_inverse=True)
    n_items = max(1, items.numel())
    key = torch.unique(rid * n_items + inv)  # ascending: by row, then by item
    del rid, inv, vals
    rid, inv = key // n_items, key % n_items
    counts = torch.bincount(inv, minlength=items.numel())
    keep = counts >= max(1, mc)
    remap = torch.cumsum(keep.to(torch.int64), 0) - 1
    sel = keep[inv]
    cols = remap[inv[sel]].to(torch.int32)
    row_len = torch.bincount(rid[sel], minlength=n_rows)
    row_ptr = torch.zeros(n_rows + 1, dtype=torch.int64, device=device)
    torch.cumsum(row_len, 0, out=row_ptr[1:])
    kept = items[keep]
    if wide:
        kept = kept ^ sign
    kept_h = kept.cpu().numpy()
    return (row_ptr, cols, (kept_h.view(np.uint64) if wide else kept_h), row_len.cpu().numpy(),
            counts[keep].cpu().numpy())


@dataclass
class _CodedInput:
    """The transactions coded on the device (``_coded_csr_device``)."""

    row_ptr: Any      # int64 [n_rows + 1], device
    codes: Any        # int32 [nnz], device: each entry's rank among the distinct ids
    col_of: Any       # int32 [n_distinct], device: the column of each code, -1 for an infrequent id
    items: np.ndarray  # the columns' ids, ascending
    row_len: np.ndarray  # each row's entries in the columns
    support: np.ndarray  # the columns' supports
    code_support: np.ndarray  # every code's support (the lex order ranks codes)


def _coded_csr_device(indptr: np.ndarray, flat: np.ndarray, n_rows: int, mc: int, device) -> _CodedInput | None:
    """The transactions coded on the device without a sort: a presence bitmap over the id span gives every id
    its rank among the distinct ids (etm_item_codes), the rows' occurrences of each rank are its support
    (etm_code_histogram), the ids with support >= mc are the columns in ascending id order, and the
    bitvectors and the row-wise kernels read the codes through the code -> column table. The same columns,
    supports and rows as ``_frequent_csr_device`` (the device input layer, gpu/input_layer.py:396-466).

    None (take ``_frequent_csr_device``) for ids that are not 64-bit signed integers within a span of
    ETM_CODE_SPAN_MAX, or when a row is not canonical (its ids unsorted or repeated), where the occurrences
    would not be supports.
    """
    import torch

    from ._lib import check, load_library

    nnz = len(flat)
    if nnz == 0 or n_rows == 0 or flat.dtype == np.uint64 or not np.issubdtype(flat.dtype, np.integer):
        return None
    vals = torch.from_numpy(np.ascontiguousarray(flat).astype(np.int64, copy=False)).to(device)
    lo_hi = torch.stack(torch.aminmax(vals)).cpu().numpy()
    lo, span = int(lo_hi[0]), int(lo_hi[1]) - int(lo_hi[0]) + 1
    if span > CODE_SPAN_MAX:
        return None
    lib = load_library()
    stream = torch.cuda.current_stream(device).cuda_stream
    n_w = -(-span // 32)
    row_ptr = torch.from_numpy(np.ascontiguousarray(indptr, dtype=np.int64)).to(device)
    bitmap = torch.empty(n_w, dtype=torch.int32, device=device)
    word_rank = torch.empty(n_w + 1, dtype=torch.int64, device=device)
    codes = torch.empty(nnz, dtype=torch.int32, device=device)
    status = torch.empty(2, dtype=torch.int32, device=device)
    check(lib.etm_item_codes(row_ptr.data_ptr(), vals.data_ptr(), nnz, n_rows, lo, span, bitmap.data_ptr(),
                             word_rank.data_ptr(), codes.data_ptr(), status.data_ptr(), stream), "etm_item_codes")
    st = status.cpu().numpy()
    n_distinct = int(word_rank[n_w].item())
    if st[0] != 0 or n_distinct < 1:
        raise RuntimeError("etm_item_codes: an id fell outside the span of the ids")
    if st[1] != 0:
        return None
    counts = torch.empty(n_distinct, dtype=torch.int64, device=device)
    check(lib.etm_code_histogram(codes.data_ptr(), nnz, n_distinct, counts.data_ptr(), stream), "etm_code_histogram")
    ids = torch.empty(n_distinct, dtype=torch.int64, device=device)
    check(lib.etm_bitmap_values(bitmap.data_ptr(), span, word_rank.data_ptr(), lo, ids.data_ptr(), stream),
          "etm_bitmap_values")
    keep = counts >= max(1, mc)
    col_of = torch.cumsum(keep.to(torch.int32), 0, dtype=torch.int32) - 1
    col_of[~keep] = -1
    code_support = counts.cpu().numpy()
    keep_h = code_support >= max(1, mc)
    return _CodedInput(row_ptr, codes, col_of, ids.cpu().numpy()[keep_h], _kept_lengths(row_ptr, codes, col_of),
                       code_support[keep_h], code_support)


def _kept_lengths(row_ptr, codes, col_of) -> np.ndarray:
    """Each row's entries whose code maps to a column (etm_kept_lengths), on the host."""
    import torch

    from ._lib import check, load_library

    n_rows = int(row_ptr.numel()) - 1
    out = torch.empty(max(1, n_rows), dtype=torch.int64, device=row_ptr.device)
    check(load_library().etm_kept_lengths(row_ptr.data_ptr(), codes.data_ptr(), n_rows, col_of.data_ptr(),
                                          col_of.numel(), out.data_ptr(),
                                          torch.cuda.current_stream(row_ptr.device).cuda_stream), "etm_kept_lengths")
    return out[:n_rows].cpu().numpy()


#: Widest id span coded through the presence bitmap (ETM_CODE_SPAN_MAX).
CODE_SPAN_MAX = 1 << 26

#: Device bytes per row the lex row order holds at its peak (two int64 keys, the sort's keys, indices and
#: buffers, the permuted lengths and offsets), plus 4 per entry for the permuted columns; without them free the
#: rows keep their order (gpu/input_layer.py:56-58, 500-529).
LEX_BYTES_PER_ROW = 96


def _lex_order(row_ptr, cols, support: np.ndarray):
    """A device CSR of columns with its rows in the lex row order (gpu/input_layer.py:408-430): sorted by the
    ranks of their most frequent columns (etm_row_order_keys, then a stable sort by the low key and one by
    the high key), the entries moved by etm_permute_rows. Rows sharing their frequent columns gather, so
    deep itemsets' rows fill few tiles and the tile occupancy skips the rest; counts do not depend on the
    order. Returns (row_ptr, cols, host row lengths), or None when the order does not fit on the device.

    Ranks follow descending support, ties by column (the reference ranks by occurrences, repeats included;
    the order differs only where a row repeats an item and never changes a count).
    """
    import torch

    from ._lib import check, load_library

    n_rows = int(row_ptr.numel()) - 1
    n_cols = len(support)
    nnz = int(cols.numel())
    dev = row_ptr.device
    if n_rows < 2 or n_cols == 0 or nnz == 0:
        return None
    free, _ = torch.cuda.mem_get_info(dev)
    if LEX_BYTES_PER_ROW * n_rows + 4 * nnz > free:
        return None
    lib = load_library()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rank = np.empty(n_cols, np.int32)
    rank[np.argsort(-np.asarray(support, np.int64), kind="stable")] = np.arange(n_cols, dtype=np.int32)
    try:
        rank_d = torch.from_numpy(rank).to(dev)
        key_hi = torch.empty(n_rows, dtype=torch.int64, device=dev)
        key_lo = torch.empty(n_rows, dtype=torch.int64, device=dev)
        check(lib.etm_row_order_keys(row_ptr.data_ptr(), cols.data_ptr(), n_rows, rank_d.data_ptr(), n_cols,
                                     key_hi.data_ptr(), key_lo.data_ptr(), stream), "etm_row_order_keys")
        order = torch.argsort(key_lo, stable=True)
        order = order[torch.argsort(key_hi[order], stable=True)]
        del key_hi, key_lo
        lens = (row_ptr[1:] - row_ptr[:-1])[order]
        new_ptr = torch.zeros(n_rows + 1, dtype=torch.int64, device=dev)
        torch.cumsum(lens, 0, out=new_ptr[1:])
        new_cols = torch.empty_like(cols)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        check(lib.etm_permute_rows(row_ptr.data_ptr(), cols.data_ptr(), nnz, order.data_ptr(), n_rows,
                                   new_ptr.data_ptr(), new_cols.data_ptr(), status.data_ptr(), stream),
              "etm_permute_rows")
        if int(status.item()) != 0:
            raise RuntimeError("etm_permute_rows: the row order is not a permutation of the rows")
        return new_ptr, new_cols, lens.cpu().numpy()
    except torch.cuda.OutOfMemoryError:
        # The free-memory check reads the device once; the sort's buffers can still miss: keep the order.
        return None


def _bitvecs_of_device_csr(row_ptr, cols, n_cols: int, n_rows: int, lut=None):
    """Column bitvectors [n_cols, ceil(N/64)] (torch int64) from a device CSR (etm_build_bitvecs); with ``lut``
    (int32, -1 for none) the entries are codes and ``lut`` their columns."""
    import torch

    from ._lib import check, load_library

    lib = load_library()
    ld = max(1, (n_rows + 63) // 64)
    bv = torch.empty((max(n_cols, 1), ld), dtype=torch.int64, device=row_ptr.device)
    ids = cols if cols.numel() else torch.zeros(1, dtype=torch.int32, device=row_ptr.device)
    check(lib.etm_build_bitvecs(row_ptr.data_ptr(), ids.data_ptr(), cols.numel(),
                                None if lut is None else lut.data_ptr(), 0 if lut is None else lut.numel(), n_rows,
                                n_cols, ld, bv.data_ptr(), torch.cuda.current_stream().cuda_stream),
          "etm_build_bitvecs")
    return bv[:n_cols]


def build_device_bitvecs(row_ptr: np.ndarray, cols: np.ndarray, n_cols: int, n_rows: int, device=None,
                         keep_rows: bool = False):
    """Column bitvectors [n_cols, ceil(N/64)] (torch int64 view of uint64) built on the device by etm_build_bitvecs.

    With ``keep_rows`` also returns the device CSR (row_ptr, cols) and the host row lengths, for the
    row-wise K=2 kernel."""
    import torch

    from ._lib import check, load_library

    lib = load_library()
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    ld = max(1, (n_rows + 63) // 64)
    rp = torch.from_numpy(row_ptr.astype(np.int64)).to(dev)
    ids = torch.from_numpy(cols.astype(np.int32)).to(dev) if len(cols) else torch.zeros(1, dtype=torch.int32, device=dev)
    bv = torch.empty((max(n_cols, 1), ld), dtype=torch.int64, device=dev)
    if len(row_ptr) != n_rows + 1 or (n_rows and np.any(np.diff(row_ptr) < 0)) or row_ptr[-1] != len(cols):
        raise ValueError("row_ptr must be a non-decreasing [n_rows + 1] array ending at len(cols)")
    check(lib.etm_build_bitvecs(rp.data_ptr(), ids.data_ptr(), len(cols), None, 0, n_rows, n_cols, ld, bv.data_ptr(),
                                torch.cuda.current_stream().cuda_stream), "etm_build_bitvecs")
    if keep_rows:
        return bv[:n_cols], (rp, ids, np.diff(row_ptr))
    return bv[:n_cols]


# ---- output ------------------------------------------------------------------------

class ItemsetFrame:
    """The result without polars or pyarrow: ``itemset`` as (offsets, values) arrays and ``support`` float64.

    ``to_arrow()`` / ``to_polars()`` convert when those libraries are
    installed; ``itemsets()`` gives the rows as tuples.
    """

    def __init__(self, offsets: np.ndarray, values: np.ndarray, support: np.ndarray):
        self.offsets = offsets
        self.values = values
        self.support = support

    def __len__(self) -> int:
        return len(self.support)

    @property
    def item_dtype(self) -> np.dtype:
        return self.values.dtype

    def itemsets(self) -> list[tuple[int, ...]]:
        v, o = self.values.tolist(), self.offsets.tolist()
        return [tuple(v[o[i]:o[i + 1]]) for i in range(len(self))]

    def to_arrow(self):
        if pa is None:
            raise ImportError("pyarrow is not installed")
        kind = self.values.dtype
        item_type = (pa.uint64() if kind == np.uint64 else pa.float64() if np.issubdtype(kind, np.floating)
                     else pa.large_string() if kind.kind in "UO" else pa.int64())
        itemset = pa.LargeListArray.from_arrays(pa.array(self.offsets, pa.int64()), pa.array(self.values, item_type))
        return pa.table({"itemset": itemset, "support": pa.array(self.support, pa.float64())})

    def to_polars(self):
        if _pl is None:
            raise ImportError("polars is not installed")
        return _pl.from_arrow(self.to_arrow())

    def __repr__(self) -> str:
        return f"ItemsetFrame({len(self)} itemsets, items {self.values.dtype})"


def _frame(levels: list[tuple[np.ndarray, np.ndarray]], n_rows: int, wide: bool):
    """itemset (list of ascending ids: Int64, UInt64 kept) + support (count / N).

    A polars DataFrame when polars is installed, else a pyarrow Table when
    pyarrow is, else an ``ItemsetFrame``.
    """
    np_type = np.uint64 if wide else np.int64
    flats, offs, sups = [], [np.zeros(1, dtype=np.int64)], []
    total = 0
    for items, counts in levels:
        n, k = items.shape
        if n == 0:
            continue
        flats.append(np.ascontiguousarray(items).astype(np_type).ravel())
        offs.append(total + k * np.arange(1, n + 1, dtype=np.int64))
        total += n * k
        sups.append(np.asarray(counts, dtype=np.float64) / max(1, n_rows))
    frame = ItemsetFrame(np.concatenate(offs), np.concatenate(flats) if flats else np.zeros(0, np_type),
                         np.concatenate(sups) if sups else np.zeros(0))
    if _pl is not None:
        return frame.to_polars()
    if pa is not None:
        return frame.to_arrow()
    return frame


def result_pairs(result, n_rows: int) -> list[tuple[tuple[int, ...], int]]:
    """A result (frame or (frame, session)) as sorted (itemset tuple, count) pairs; count = rint(support * N)."""
    df = result[0] if isinstance(result, tuple) else result
    if isinstance(df, ItemsetFrame):
        sets, sup = df.itemsets(), df.support
    else:
        table = df if (pa is not None and isinstance(df, pa.Table)) else df.to_arrow()
        sets = [tuple(s) for s in table.column("itemset").to_pylist()]
        sup = np.asarray(table.column("support").to_numpy(), dtype=np.float64)
    counts = np.rint(np.asarray(sup, dtype=np.float64) * n_rows).astype(np.int64)

    def item(x):
        return int(x) if isinstance(x, (numbers.Integral, np.integer)) else (float(x) if isinstance(x, float) else x)

    out = [(tuple(item(x) for x in s), int(c)) for s, c in zip(sets, counts)]
    out.sort(key=lambda t: (len(t[0]), t[0]))
    return out


def _array_facts(bv) -> tuple[tuple[int, ...], str, bool]:
    """(shape, numpy typestr, C-contiguous) of a device array: a torch CUDA tensor or any
    ``__cuda_array_interface__`` object (core/apriori.py:491-527 checks the same facts)."""
    try:
        import torch

        if isinstance(bv, torch.Tensor):
            if not bv.is_cuda:
                raise TypeError("bitvecs_gpu must be a CUDA tensor")
            typestr = {torch.uint64: "<u8", torch.int64: "<i8"}.get(bv.dtype, str(bv.dtype))
            return tuple(bv.shape), typestr, bv.is_contiguous()
    except ImportError:  # pragma: no cover
        pass
    cai = getattr(bv, "__cuda_array_interface__", None)
    if cai is None:
        raise TypeError(f"bitvecs_gpu must expose __cuda_array_interface__, got {type(bv).__name__}")
    shape = tuple(cai["shape"])
    strides = cai.get("strides")
    contiguous = strides is None or (len(shape) == 2 and tuple(strides) == (shape[1] * 8, 8))
    return shape, cai["typestr"], contiguous


def _emit(out: MineOutput, col_items: np.ndarray, labels: np.ndarray | None = None):
    """The result frame; item ids, offsets and supports are built on the device (``frame_arrays``). With
    ``labels``, the ids are codes of non-integer items and map back through them."""
    offsets, values, support, _ = out.frame_arrays(col_items)
    if labels is not None:
        values = labels[values]
    frame = ItemsetFrame(offsets, values, support)
    if _pl is not None:
        return frame.to_polars()
    if pa is not None:
        return frame.to_arrow()
    return frame


class _LevelFlush:
    """The per-level parquet flush (``io/flush.py:63-140`` driven from ``gpu/row_split.py:511-535``): each
    final level goes to ``frequent_k{k}.parquet`` on a writer thread while the device counts the next
    one. At most two levels wait for the writer; ``close`` waits for every write and raises its error."""

    def __init__(self, output_dir: str, item_of_col: np.ndarray, n_rows: int):
        self.dir = output_dir
        self.items = item_of_col
        self.n = max(1, n_rows)
        self.pool = ThreadPoolExecutor(1, thread_name_prefix="etm-flush")
        self.pending: list = []

    def __call__(self, k: int, cols: np.ndarray, counts: np.ndarray) -> None:
        while len(self.pending) >= 2:
            self.pending.pop(0).result()
        items = self.items[cols]
        sup = counts.astype(np.float64) / self.n
        self.pending.append(self.pool.submit(_flush.write_level, _flush.level_path(self.dir, k), items, sup))

    def close(self) -> None:
        try:
            for f in self.pending:
                f.result()
        finally:
            self.pending = []
            self.pool.shutdown(wait=True)


def _check_flush_options(output_dir, resume_from_k) -> bool:
    """Validate output_dir / resume_from_k; True when the mine resumes (``gpu/row_split.py:540``: K >= 2 with
    an output directory; resume_from_k=1 mines from the start)."""
    if output_dir is not None:
        if not isinstance(output_dir, (str, os.PathLike)):
            raise TypeError(f"output_dir must be a path, got {type(output_dir).__name__}")
        if "://" in os.fspath(output_dir):
            raise ValueError(f"output_dir={output_dir!r}: only a local directory is supported (no object-store upload)")
    if resume_from_k is None:
        return False
    if isinstance(resume_from_k, bool) or not isinstance(resume_from_k, numbers.Integral) or resume_from_k < 1:
        raise ValueError(f"resume_from_k must be a positive integer, got {resume_from_k!r}")
    if output_dir is None:
        raise ValueError("resume_from_k needs output_dir: the level to resume from is read from "
                         "output_dir/frequent_k{resume_from_k}.parquet")
    return resume_from_k >= 2


def _resume_level(output_dir: str, k: int, item_of_col: np.ndarray, n_rows: int):
    """(k, caller columns [n, k], counts [n]) of the flushed level k: item ids map to columns, counts come back
    as rint(support * N), exact for any int32 count (``gpu/row_split.py:546-606``)."""
    path = _flush.level_path(output_dir, k)
    if not path.exists():
        raise FileNotFoundError(f"resume_from_k={k}: {path} does not exist")
    itemsets, sup = _flush.read_level(path)
    if len(sup) and itemsets.shape[1] != k:
        raise ValueError(f"{path} holds itemsets of length {itemsets.shape[1]}, not {k}")
    flat = itemsets.reshape(-1)
    order = np.argsort(item_of_col, kind="stable")
    ids = item_of_col[order]
    if flat.size:
        if item_of_col.dtype == np.uint64:
            if flat.dtype.kind == "i" and (flat < 0).any():
                raise ValueError(f"{path} holds item ids that are not in this input")
            flat = flat.astype(np.uint64)
        else:
            flat = flat.astype(np.int64)
        pos = np.minimum(np.searchsorted(ids, flat), max(0, len(ids) - 1))
        if len(ids) == 0 or (ids[pos] != flat).any():
            raise ValueError(f"{path} holds item ids that are not in this input")
        cols = order[pos].astype(np.int64).reshape(-1, k)
    else:
        cols = np.zeros((0, k), np.int64)
    counts = np.rint(sup.astype(np.float64) * n_rows).astype(np.int64)
    return k, cols, counts


def _mine_to(eng: Engine, bv, n_rows: int, min_support: float, max_length, item_of_col: np.ndarray,
             output_dir, resume_from_k, **kw) -> MineOutput:
    """One mine, with the per-level flush and resume when output_dir is given."""
    if output_dir is None:
        return eng.mine(bv, n_rows, min_support, max_length, **kw)
    os.makedirs(output_dir, exist_ok=True)
    resume = _resume_level(output_dir, int(resume_from_k), item_of_col, n_rows) if resume_from_k else None
    writer = _LevelFlush(os.fspath(output_dir), item_of_col, n_rows)
    try:
        return eng.mine(bv, n_rows, min_support, max_length, on_level=writer, resume=resume, keep_levels=False,
                        **kw)
    finally:
        writer.close()


def _session_from(out: MineOutput, session: ProfilingSession) -> None:
    for s in out.stats:
        session.record_phase(f"k{s.k}", s.ms, n_candidates=s.n_candidates, n_frequent=s.n_frequent,
                             n_groups=s.n_groups, n_chunks=s.n_chunks)


def apriori(
    transactions=None,
    min_support: float = 0.5,
    max_length: int | None = None,
    item_col: str = "items",
    use_gpu: bool = False,
    batch_size: int | None = 10_000,
    profile: bool = False,
    show_progress: bool = False,
    warn_complexity: bool = True,
    prune_equal_support: bool = False,
    use_generator_pruning: bool = False,
    prune_apriori: bool = True,
    sparse: bool | None = None,
    n_jobs: int = 1,
    enable_length_filter: bool = True,
    streaming: bool = False,
    chunk_size: int = 10_000_000,
    n_gpus: int = 1,
    memory_budget_gb: float | None = None,
    progress_callback=None,
    level_callback=None,
    gpu_resident: bool = False,
    bitvecs: tuple | None = None,
    output_dir: str | None = None,
    resume_from_k: int | None = None,
    max_ram_gb: float = 800.0,
    max_vram_gb: float = 70.0,
    sparse_from_k: int | str | None = None,
    anchor_items: set | None = None,
    *,
    engine: Engine | None = None,
) -> Any:
    """Frequent itemsets (or free-sets) with exact counts, mined on one GB300.

    Parameters mean what they mean on the reference's ``apriori``; see the
    module docstring for the inputs served. ``engine`` (keyword only, an
    extension) reuses an ``Engine`` and its device scratch across calls.
    """
    _validate_parameters(min_support, max_length, batch_size, sparse_from_k, prune_apriori)
    if sparse is not None:
        raise ValueError("sparse= was removed: no route reads it. Drop the argument.")
    if gpu_resident:
        raise ValueError("gpu_resident was removed: use_gpu=True (or bitvecs=) keeps candidates and counts on the GPU.")
    _unsupported(
        streaming=(streaming, "SON streaming is not this engine's path"),
        anchor_items=(anchor_items is not None, "anchor filtering is not built"),
        memory_budget_gb=(memory_budget_gb is not None, "it only sizes SON chunks"),
        n_gpus=(n_gpus != 1, "one GB300 per call; run independent calls per GPU"),
    )
    if bitvecs is None and not use_gpu:
        raise ValueError("the GB300 engine serves the GPU route: pass use_gpu=True or bitvecs=")
    resuming = _check_flush_options(output_dir, resume_from_k)
    resume_k = resume_from_k if resuming else None
    session = ProfilingSession() if profile else None

    if bitvecs is not None:
        if transactions is not None:
            raise ValueError("Cannot provide both 'transactions' and 'bitvecs'.")
        if not isinstance(bitvecs, tuple) or len(bitvecs) != 3:
            raise ValueError("bitvecs must be a tuple of (bitvecs_gpu, col_to_item, n_transactions)")
        bv, col_to_item, n_trans = bitvecs
        shape, typestr, contiguous = _array_facts(bv)
        if len(shape) != 2:
            raise ValueError(f"bitvecs_gpu must be 2D (n_cols, n_u64s), got {len(shape)}D")
        if isinstance(n_trans, bool) or not isinstance(n_trans, numbers.Integral) or n_trans < 0:
            raise ValueError(f"n_transactions must be a non-negative integer, got {n_trans!r}")
        expected = math.ceil(n_trans / 64)
        if shape[1] != expected:
            raise ValueError(f"bitvecs_gpu.shape[1] ({shape[1]}) must equal ceil(n_transactions/64) = {expected}")
        if len(col_to_item) != shape[0]:
            raise ValueError(f"col_to_item has {len(col_to_item)} keys but bitvecs_gpu has {shape[0]} columns")
        if not all(isinstance(v, numbers.Integral) for v in col_to_item.values()):
            raise ValueError("col_to_item must map every column to an integer item id")
        if typestr not in ("<u8", "|u8") or not contiguous:
            raise ValueError(f"bitvecs_gpu must be a C-contiguous uint64 array, got {typestr}, c_contiguous={contiguous}")
        n_trans = int(n_trans)
        if n_trans > np.iinfo(np.int32).max:
            raise ValueError(f"n_transactions={n_trans:,} exceeds int32 max: the count arrays are int32")
        vals = [int(col_to_item[c]) for c in range(shape[0])] if shape[0] else []
        wide = any(v > np.iinfo(np.int64).max for v in vals)
        col_items = np.array(vals, dtype=np.uint64 if wide else np.int64)
        eng = engine or Engine()
        out = _mine_to(eng, bv, n_trans, min_support, max_length, col_items, output_dir, resume_k,
                       prune_equal_support=prune_equal_support, use_generator_pruning=use_generator_pruning,
                       level_callback=level_callback,
                       n_cols_logical=(max(col_to_item.keys()) + 1) if col_to_item else 0,
                       max_ram_gb=max_ram_gb, max_vram_gb=max_vram_gb)
        if warn_complexity and out.stats:
            _warn_complexity(out.stats[0].n_frequent, min_support)
        # With output_dir the levels are in the files; the frame is empty (gpu/row_split.py:1172-1178).
        df = _emit(out, col_items) if output_dir is None else _frame([], max(1, n_trans), wide)
        if session is not None:
            _session_from(out, session)
        return (df, session) if profile else df

    if transactions is None:
        raise ValueError("Either 'transactions' or 'bitvecs' must be provided")
    indptr, flat, kind, labels = _list_column(transactions, item_col)
    if labels is not None and (output_dir is not None or resume_from_k is not None):
        raise ValueError("output_dir and resume_from_k store integer item ids: these items are not integer ids")
    eng = engine or Engine()
    n_rows = len(indptr) - 1
    if n_rows > np.iinfo(np.int32).max:
        raise ValueError(f"n_transactions={n_rows:,} exceeds int32 max")
    wide = np.dtype(kind) == np.uint64
    mc = min_count(min_support, n_rows)
    coded = _coded_csr_device(indptr, flat, n_rows, mc, eng.device)
    if coded is not None:
        # Entries hold codes; col_of maps them to the columns.
        row_ptr, cols, items, row_len, col_of = coded.row_ptr, coded.codes, coded.items, coded.row_len, coded.col_of
        rank_support = np.where(coded.code_support >= max(1, mc), coded.code_support, -1)
    else:
        row_ptr, cols, items, row_len, rank_support = _frequent_csr_device(indptr, flat, n_rows, mc, eng.device)
        col_of = None
    if len(items) == 0:
        df = _frame([], max(1, n_rows), wide)
        return (df, session) if profile else df
    # The lex row order, and with it the tile-occupancy skip (core/apriori.py:627-640, gpu/row_split.py:397-413).
    lex = (_lex_order(row_ptr, cols, rank_support) if eng.row_order == "lex" and n_rows >= eng.lex_min_rows
           else None)
    if lex is not None:
        row_ptr, cols, row_len = lex
        if col_of is not None:
            row_len = _kept_lengths(row_ptr, cols, col_of)  # the rows' entries in the columns, in the new order
    bv = _bitvecs_of_device_csr(row_ptr, cols, len(items), n_rows, col_of)
    rows = (row_ptr, cols, row_len) if col_of is None else (row_ptr, cols, row_len, col_of)
    max_tx = int(np.diff(indptr).max()) if n_rows else 0
    eff = min(max_length, max_tx) if max_length else max_tx
    col_items = items.astype(np.uint64 if wide else np.int64)
    out = _mine_to(eng, bv, n_rows, min_support, eff if eff >= 1 else 1, col_items, output_dir, resume_k,
                   prune_equal_support=prune_equal_support, use_generator_pruning=use_generator_pruning,
                   level_callback=level_callback, rows=rows, max_ram_gb=max_ram_gb, max_vram_gb=max_vram_gb,
                   occupancy=lex is not None)
    if warn_complexity and out.stats:
        _warn_complexity(out.stats[0].n_frequent, min_support)
    df = _emit(out, col_items, labels) if output_dir is None else _frame([], max(1, n_rows), wide)
    if session is not None:
        _session_from(out, session)
    return (df, session) if profile else df
