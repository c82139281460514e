"""Per-level parquet flush and its reader: ``frequent_k{k}.parquet`` as the reference writes it.

Each level is one file with two columns (``io/flush.py:63-140``): ``itemset``,
a large list of the level's item ids (int32 when every id fits, else int64;
UInt64 ids are kept as unsigned), and ``support`` (Float64 = count / N). The
reference writes them with pyarrow (zstd, level 2, no dictionary); here pyarrow
is used the same way when it is installed. Without it (the GPU machine has none) a
small built-in codec writes and reads the same schema: one row group, PLAIN
values, levels in the RLE / bit-packed hybrid, Thrift compact-protocol
metadata, gzip or no compression. Files of either writer open in pyarrow, and
the built-in reader reads its own files and pyarrow's uncompressed or gzip ones
(zstd needs pyarrow).

Resume (``gpu/row_split.py:546-606``) reads a level back and rebuilds its
counts as rint(support * N), exact for any int32 count.
"""

from __future__ import annotations

import gzip
import os
import struct
from pathlib import Path

import numpy as np

try:  # optional: the reference's writer
    import pyarrow as _pa
    import pyarrow.parquet as _pq
except Exception:  # pragma: no cover - the GPU machine has no pyarrow
    _pa = None
    _pq = None


def level_path(output_dir: str | os.PathLike, k: int) -> Path:
    return Path(output_dir) / f"frequent_k{k}.parquet"


def _item_array(itemsets: np.ndarray) -> np.ndarray:
    """Item ids as the flush stores them: int32 when every id fits (the reference's large_list<int32>),
    else int64, UInt64 kept."""
    a = np.ascontiguousarray(itemsets)
    if a.dtype == np.uint64:
        return a
    a = a.astype(np.int64, copy=False)
    if a.size == 0 or (a.min() >= np.iinfo(np.int32).min and a.max() <= np.iinfo(np.int32).max):
        return a.astype(np.int32)
    return a


def write_level(path: str | os.PathLike, itemsets: np.ndarray, supports: np.ndarray, *,
                engine: str | None = None, compression: str = "zstd") -> Path:
    """Write one level: ``itemsets`` [n, k] item ids, ``supports`` float64 [n]. ``engine`` "pyarrow" or
    "builtin" (default: pyarrow when installed); the built-in codec writes gzip for a compression it lacks."""
    path = Path(path)
    items = _item_array(itemsets)
    n = len(supports)
    k = items.shape[1] if items.ndim == 2 else 1
    sup = np.ascontiguousarray(supports, dtype=np.float64)
    use_arrow = (engine or ("pyarrow" if _pq is not None else "builtin")) == "pyarrow"
    tmp = path.with_suffix(path.suffix + ".tmp")
    if use_arrow:
        if _pq is None:
            raise ImportError("pyarrow is not installed")
        offsets = np.arange(0, (n + 1) * k, k, dtype=np.int64)
        table = _pa.table({"itemset": _pa.LargeListArray.from_arrays(offsets, items.ravel()),
                           "support": sup})
        kw = {"compression": compression, "use_dictionary": False}
        if compression == "zstd":
            kw["compression_level"] = 2
        _pq.write_table(table, str(tmp), **kw)
    else:
        tmp.write_bytes(_Writer(items.reshape(n, k), sup, "gzip" if compression not in ("none", None) else "none")
                        .file_bytes())
    os.replace(tmp, path)
    return path


def read_level(path: str | os.PathLike, *, engine: str | None = None) -> tuple[np.ndarray, np.ndarray]:
    """(itemsets [n, k] item ids, supports float64 [n]) of one flushed level."""
    path = Path(path)
    if (engine or ("pyarrow" if _pq is not None else "builtin")) == "pyarrow":
        if _pq is None:
            raise ImportError("pyarrow is not installed")
        table = _pq.read_table(str(path))
        col = table.column("itemset").combine_chunks()
        values = col.values.to_numpy(zero_copy_only=False)
        offsets = np.asarray(col.offsets.to_numpy(zero_copy_only=False), dtype=np.int64)
        sup = table.column("support").combine_chunks().to_numpy(zero_copy_only=False).astype(np.float64)
    else:
        offsets, values, sup = _read_builtin(path.read_bytes())
    n = len(sup)
    if n == 0:
        return np.zeros((0, 0), dtype=values.dtype if len(values) else np.int64), sup
    lens = np.diff(offsets)
    if not (lens == lens[0]).all():
        raise ValueError(f"{path}: itemsets of different lengths in one level")
    return np.asarray(values).reshape(n, int(lens[0])), sup


# ---- the built-in codec ---------------------------------------------------------------------------------------
# Thrift compact protocol: field headers (delta << 4 | type), zigzag varints, lists (size << 4 | elem type).
_I32, _I64, _BINARY, _LIST, _STRUCT = 5, 6, 8, 9, 12
# Parquet enums.
_T_INT32, _T_INT64, _T_DOUBLE = 1, 2, 5
_REQUIRED, _REPEATED = 0, 2
_LIST_CONVERTED, _UINT_64 = 3, 14
_PLAIN, _RLE = 0, 3
_CODEC = {"none": 0, "gzip": 2}


def _varint(v: int) -> bytes:
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _zigzag(v: int) -> int:
    return (v << 1) ^ (v >> 63)


class _Struct:
    """A Thrift compact struct being written: fields in increasing id order."""

    def __init__(self):
        self.buf = bytearray()
        self.last = 0

    def _head(self, fid: int, ftype: int) -> None:
        delta = fid - self.last
        if 0 < delta <= 15:
            self.buf.append((delta << 4) | ftype)
        else:
            self.buf.append(ftype)
            self.buf += _varint(_zigzag(fid))
        self.last = fid

    def i32(self, fid: int, v: int) -> "_Struct":
        self._head(fid, _I32)
        self.buf += _varint(_zigzag(v))
        return self

    def i64(self, fid: int, v: int) -> "_Struct":
        self._head(fid, _I64)
        self.buf += _varint(_zigzag(v))
        return self

    def string(self, fid: int, s: str) -> "_Struct":
        b = s.encode()
        self._head(fid, _BINARY)
        self.buf += _varint(len(b)) + b
        return self

    def struct(self, fid: int, inner: "_Struct") -> "_Struct":
        self._head(fid, _STRUCT)
        self.buf += inner.end()
        return self

    def list(self, fid: int, elem_type: int, items: list) -> "_Struct":
        self._head(fid, _LIST)
        n = len(items)
        self.buf.append((n << 4) | elem_type if n < 15 else 0xF0 | elem_type)
        if n >= 15:
            self.buf += _varint(n)
        for it in items:
            if elem_type == _STRUCT:
                self.buf += it.end()
            elif elem_type == _I32:
                self.buf += _varint(_zigzag(it))
            elif elem_type == _BINARY:
                b = it.encode()
                self.buf += _varint(len(b)) + b
        return self

    def end(self) -> bytes:
        return bytes(self.buf) + b"\x00"


def _bitpacked_levels(levels: np.ndarray) -> bytes:
    """Levels of bit width 1 as one bit-packed run of the RLE / bit-packed hybrid, with its 4-byte length."""
    n = len(levels)
    groups = (n + 7) // 8
    padded = np.zeros(groups * 8, np.uint8)
    padded[:n] = levels
    data = _varint((groups << 1) | 1) + np.packbits(padded, bitorder="little").tobytes()
    return struct.pack("<I", len(data)) + data


class _Writer:
    def __init__(self, items: np.ndarray, sup: np.ndarray, codec: str):
        self.items, self.sup, self.codec = items, sup, codec

    def _page(self, num_values: int, body: bytes, levels: bool) -> tuple[bytes, int, int]:
        # Level 1: the fast end, like the reference's zstd level 2 (a level can be megabytes to gigabytes).
        payload = gzip.compress(body, compresslevel=1) if self.codec == "gzip" else body
        dph = _Struct().i32(1, num_values).i32(2, _PLAIN).i32(3, _RLE).i32(4, _RLE)
        header = _Struct().i32(1, 0).i32(2, len(body)).i32(3, len(payload)).struct(5, dph).end()
        return header + payload, len(header) + len(body), len(header) + len(payload)

    def file_bytes(self) -> bytes:
        n, k = self.items.shape
        vals = self.items.ravel()
        phys = _T_INT32 if vals.dtype == np.int32 else _T_INT64
        out = bytearray(b"PAR1")
        # itemset.list.element: repetition level 0 at each itemset's first item, 1 after; every value defined.
        rep = np.ones(n * k, np.uint8)
        rep[::max(k, 1)] = 0
        body = _bitpacked_levels(rep) + _bitpacked_levels(np.ones(n * k, np.uint8)) + \
            vals.astype(vals.dtype.newbyteorder("<")).tobytes()
        page, usize, csize = self._page(n * k, body, True)
        off_items = len(out)
        out += page
        cm_items = (_Struct().i32(1, phys).list(2, _I32, [_PLAIN, _RLE])
                    .list(3, _BINARY, ["itemset", "list", "element"]).i32(4, _CODEC[self.codec])
                    .i64(5, n * k).i64(6, usize).i64(7, csize).i64(9, off_items))
        page, usize2, csize2 = self._page(n, self.sup.astype("<f8").tobytes(), False)
        off_sup = len(out)
        out += page
        cm_sup = (_Struct().i32(1, _T_DOUBLE).list(2, _I32, [_PLAIN]).list(3, _BINARY, ["support"])
                  .i32(4, _CODEC[self.codec]).i64(5, n).i64(6, usize2).i64(7, csize2).i64(9, off_sup))
        element = _Struct().i32(1, phys).i32(3, _REQUIRED).string(4, "element")
        if vals.dtype == np.uint64:
            element.i32(6, _UINT_64)
        schema = [
            _Struct().string(4, "schema").i32(5, 2),
            _Struct().i32(3, _REQUIRED).string(4, "itemset").i32(5, 1).i32(6, _LIST_CONVERTED),
            _Struct().i32(3, _REPEATED).string(4, "list").i32(5, 1),
            element,
            _Struct().i32(1, _T_DOUBLE).i32(3, _REQUIRED).string(4, "support"),
        ]
        columns = [_Struct().i64(2, off_items).struct(3, cm_items), _Struct().i64(2, off_sup).struct(3, cm_sup)]
        row_group = _Struct().list(1, _STRUCT, columns).i64(2, usize + usize2).i64(3, n)
        meta = (_Struct().i32(1, 1).list(2, _STRUCT, schema).i64(3, n).list(4, _STRUCT, [row_group])
                .string(6, "et-miner-gb300 flush")).end()
        out += meta + struct.pack("<I", len(meta)) + b"PAR1"
        return bytes(out)


class _Reader:
    """A Thrift compact-protocol reader: structs as {field id: value}."""

    def __init__(self, buf: bytes, pos: int = 0):
        self.buf, self.pos = buf, pos

    def varint(self) -> int:
        shift = out = 0
        while True:
            b = self.buf[self.pos]
            self.pos += 1
            out |= (b & 0x7F) << shift
            if not b & 0x80:
                return out
            shift += 7

    def zz(self) -> int:
        v = self.varint()
        return (v >> 1) ^ -(v & 1)

    def value(self, t: int):
        if t in (1, 2):
            return t == 1
        if t == 3:
            self.pos += 1
            return self.buf[self.pos - 1]
        if t in (4, 5, 6):
            return self.zz()
        if t == 7:
            self.pos += 8
            return struct.unpack_from("<d", self.buf, self.pos - 8)[0]
        if t == _BINARY:
            n = self.varint()
            self.pos += n
            return bytes(self.buf[self.pos - n:self.pos])
        if t in (_LIST, 10):
            h = self.buf[self.pos]
            self.pos += 1
            n, et = h >> 4, h & 0x0F
            if n == 15:
                n = self.varint()
            return [self.value(et) for _ in range(n)]
        if t == _STRUCT:
            return self.struct()
        raise ValueError(f"unsupported thrift type {t}")

    def struct(self) -> dict:
        out, last = {}, 0
        while True:
            h = self.buf[self.pos]
            self.pos += 1
            if h == 0:
                return out
            delta, t = h >> 4, h & 0x0F
            fid = last + delta if delta else self.zz()
            out[fid] = self.value(t)
            last = fid


def _hybrid(buf: bytes, pos: int, end: int, width: int, n: int) -> np.ndarray:
    """Decode n levels of the RLE / bit-packed hybrid in buf[pos:end]."""
    out = np.empty(n, np.int64)
    got = 0
    r = _Reader(buf, pos)
    nbytes = (width + 7) // 8
    while got < n and r.pos < end:
        h = r.varint()
        if h & 1:
            count = (h >> 1) * 8
            raw = np.frombuffer(buf, np.uint8, (h >> 1) * width, r.pos)
            r.pos += (h >> 1) * width
            bits = np.unpackbits(raw, bitorder="little").reshape(-1, width)
            vals = (bits * (1 << np.arange(width))).sum(axis=1)
        else:
            count = h >> 1
            v = int.from_bytes(buf[r.pos:r.pos + nbytes], "little")
            r.pos += nbytes
            vals = np.full(count, v, np.int64)
        take = min(count, n - got)
        out[got:got + take] = vals[:take]
        got += take
    return out


def _read_builtin(data: bytes):
    if data[:4] != b"PAR1" or data[-4:] != b"PAR1":
        raise ValueError("not a parquet file")
    mlen = struct.unpack_from("<I", data, len(data) - 8)[0]
    meta = _Reader(data, len(data) - 8 - mlen).struct()
    schema = meta[2]
    by_path = {}
    leaves = {}
    # Leaves and their max levels, walking the schema tree.
    stack = [(schema[0].get(5, 0), [], 0, 0)]
    idx = 1
    while idx < len(schema):
        children, path, dl, rl = stack[-1]
        el = schema[idx]
        idx += 1
        name = el[4].decode()
        rep = el.get(3, _REQUIRED)
        d = dl + (1 if rep != _REQUIRED else 0)
        r = rl + (1 if rep == _REPEATED else 0)
        stack[-1] = (children - 1, path, dl, rl)
        if el.get(5):
            stack.append((el[5], path + [name], d, r))
        else:
            leaves[tuple(path + [name])] = (el.get(1), d, r, el.get(6))
        while stack and stack[-1][0] == 0 and len(stack) > 1:
            stack.pop()
    if len(meta[4]) != 1:
        raise ValueError("the built-in reader takes one row group")
    for col in meta[4][0][1]:
        cm = col[3]
        by_path[tuple(p.decode() for p in cm[3])] = cm
    out = {}
    for path, cm in by_path.items():
        phys, max_d, max_r, conv = leaves[path]
        codec = cm[4]
        if codec not in (0, 2):
            raise ValueError(f"compression codec {codec} needs pyarrow")
        pos = cm[9]
        remaining = cm[5]
        reps, defs, vals = [], [], []
        while remaining > 0:
            r = _Reader(data, pos)
            ph = r.struct()
            start = r.pos
            page = data[start:start + ph[3]]
            pos = start + ph[3]
            if ph[1] != 0:
                continue  # dictionary or index pages: not written without dictionaries
            body = gzip.decompress(page) if codec == 2 else page
            nv = ph[5][1]
            if ph[5][2] != _PLAIN:
                raise ValueError("only PLAIN-encoded values are supported without pyarrow")
            p = 0
            rl = np.zeros(nv, np.int64)
            dl = np.full(nv, max_d, np.int64)
            if max_r:
                ln = struct.unpack_from("<I", body, p)[0]
                rl = _hybrid(body, p + 4, p + 4 + ln, max(1, int(max_r).bit_length()), nv)
                p += 4 + ln
            if max_d:
                ln = struct.unpack_from("<I", body, p)[0]
                dl = _hybrid(body, p + 4, p + 4 + ln, max(1, int(max_d).bit_length()), nv)
                p += 4 + ln
            present = int((dl == max_d).sum())
            dt = {_T_INT32: "<i4", _T_INT64: "<u8" if conv == _UINT_64 else "<i8", _T_DOUBLE: "<f8"}[phys]
            vals.append(np.frombuffer(body, dt, present, p))
            reps.append(rl)
            defs.append(dl)
            remaining -= nv
        if not vals:  # an empty level: no pages
            dt = {_T_INT32: "<i4", _T_INT64: "<u8" if conv == _UINT_64 else "<i8", _T_DOUBLE: "<f8"}[phys]
            reps, defs, vals = [np.zeros(0, np.int64)], [np.zeros(0, np.int64)], [np.zeros(0, dt)]
        out[path] = (np.concatenate(reps), np.concatenate(defs), np.concatenate(vals), max_d)
    item_path = next(p for p in out if p[0] == "itemset")
    rl, dl, values, max_d = out[item_path]
    if (dl != max_d).any():
        raise ValueError("null itemsets or items are not supported without pyarrow")
    starts = np.flatnonzero(rl == 0)
    offsets = np.append(starts, len(rl)).astype(np.int64)
    sup = out[("support",)][2].astype(np.float64)
    return offsets, values.astype(values.dtype.newbyteorder("=")), sup
