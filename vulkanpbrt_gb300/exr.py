"""Minimal OpenEXR reader and writer for the offline replay files.

The reference reads and writes its recorded G-buffers and illumination as
OpenEXR through vsgXchange's openexr plugin (source/io/RenderIO.cpp:15,
83, 221, 557, 603). This module implements the published OpenEXR 2 file
layout for what those files use: single-part scanline images, channels of
type UINT / HALF / FLOAT with sampling 1, and the compressions NONE, RLE,
ZIPS and ZIP (zlib through Python's standard library). Other compressions
(PIZ, PXR24, B44, DWA), tiled, deep and multi-part files raise ExrError.

Layout written (and expected): magic 20000630, version 2; header attributes
channels, compression, dataWindow, displayWindow, lineOrder (increasing y),
pixelAspectRatio, screenWindowCenter, screenWindowWidth; a table of chunk
offsets; chunks of (y, byte count, data) with per-scanline, per-channel
(alphabetical) little-endian samples. RLE and ZIP data are first split into
even and odd bytes and delta-encoded (+128), as the format defines; a chunk
whose compressed form is not smaller is stored raw.

Arrays: an image is returned as a dict {channel name: [H, W] array} by
`read`; `load` shapes it as the reference's vsg data: R,G,B(,A) -> [H, W, 4]
(A = 1 when absent), two channels -> [H, W, 2], one channel -> [H, W].
"""
from __future__ import annotations

import struct
import zlib
from typing import Dict

import numpy as np

MAGIC = 20000630
UINT, HALF, FLOAT = 0, 1, 2
_DTYPE = {UINT: np.dtype("<u4"), HALF: np.dtype("<f2"), FLOAT: np.dtype("<f4")}
COMPRESSION = {"NONE": 0, "RLE": 1, "ZIPS": 2, "ZIP": 3, "PIZ": 4, "PXR24": 5, "B44": 6, "B44A": 7, "DWAA": 8,
               "DWAB": 9}
_LINES = {0: 1, 1: 1, 2: 1, 3: 16, 4: 32, 5: 16, 6: 32, 7: 32, 8: 32, 9: 256}


class ExrError(ValueError):
    pass


# ---- byte preprocessing shared by RLE and ZIP ------------------------------
def _split_predict(raw: bytes) -> np.ndarray:
    a = np.frombuffer(raw, np.uint8)
    t = np.concatenate([a[0::2], a[1::2]])
    out = t.copy()
    out[1:] = ((t[1:].astype(np.int16) - t[:-1].astype(np.int16) + 128) & 0xFF).astype(np.uint8)
    return out


def _unpredict_merge(buf: np.ndarray) -> bytes:
    d = buf.astype(np.int64)
    d[1:] -= 128
    t = (np.cumsum(d) & 0xFF).astype(np.uint8)
    n = len(t)
    h = (n + 1) // 2
    out = np.empty(n, np.uint8)
    out[0::2] = t[:h]
    out[1::2] = t[h:]
    return out.tobytes()


def _rle_encode(a: np.ndarray) -> bytes:
    out = bytearray()
    n, i = len(a), 0
    while i < n:
        j = i + 1
        while j < n and a[j] == a[i] and j - i < 128:
            j += 1
        if j - i >= 3:  # a run: count - 1, value
            out += struct.pack("<b", j - i - 1)
            out.append(int(a[i]))
            i = j
            continue
        k = i  # a literal stretch up to the next run of three
        while k < n and k - i < 127 and not (k + 2 < n and a[k] == a[k + 1] == a[k + 2]):
            k += 1
        out += struct.pack("<b", -(k - i))
        out += a[i:k].tobytes()
        i = k
    return bytes(out)


def _rle_decode(data: bytes, expected: int) -> np.ndarray:
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        c = struct.unpack_from("<b", data, i)[0]
        i += 1
        if c < 0:
            out += data[i:i - c]
            i -= c
        else:
            if i >= n:
                raise ExrError("truncated RLE data")
            out += bytes([data[i]]) * (c + 1)
            i += 1
    if len(out) != expected:
        raise ExrError(f"RLE data decodes to {len(out)} bytes, expected {expected}")
    return np.frombuffer(bytes(out), np.uint8)


def _compress(raw: bytes, comp: int) -> bytes:
    if comp == 0:
        return raw
    pre = _split_predict(raw)
    if comp == 1:
        return _rle_encode(pre)
    return zlib.compress(pre.tobytes())


def _decompress(data: bytes, comp: int, expected: int) -> bytes:
    if comp == 0 or len(data) == expected:
        return data
    if comp == 1:
        return _unpredict_merge(_rle_decode(data, expected))
    if comp in (2, 3):
        pre = zlib.decompress(data)
        if len(pre) != expected:
            raise ExrError(f"ZIP data decodes to {len(pre)} bytes, expected {expected}")
        return _unpredict_merge(np.frombuffer(pre, np.uint8))
    name = {v: k for k, v in COMPRESSION.items()}.get(comp, str(comp))
    raise ExrError(f"EXR compression {name} is not supported (NONE, RLE, ZIPS, ZIP are)")


# ---- header ----------------------------------------------------------------
def _cstr(buf: bytes, pos: int):
    end = buf.index(b"\0", pos)
    return buf[pos:end].decode("latin-1"), end + 1


def _parse_header(buf: bytes):
    if len(buf) < 8 or struct.unpack_from("<i", buf, 0)[0] != MAGIC:
        raise ExrError("not an OpenEXR file")
    version = struct.unpack_from("<i", buf, 4)[0]
    if version & 0xFF != 2:
        raise ExrError(f"unsupported EXR version {version & 0xFF}")
    if version & (0x200 | 0x800 | 0x1000):
        raise ExrError("tiled, deep and multi-part EXR files are not supported")
    pos = 8
    attrs = {}
    while True:
        name, pos = _cstr(buf, pos)
        if not name:
            break
        typ, pos = _cstr(buf, pos)
        size = struct.unpack_from("<i", buf, pos)[0]
        pos += 4
        attrs[name] = (typ, buf[pos:pos + size])
        pos += size
    for req in ("channels", "compression", "dataWindow"):
        if req not in attrs:
            raise ExrError(f"EXR header lacks {req}")
    chans = []
    raw = attrs["channels"][1]
    p = 0
    while p < len(raw) and raw[p] != 0:
        cname, p = _cstr(raw, p)
        ptype, _plin, xs, ys = struct.unpack_from("<iB3xii", raw, p)
        p += 16
        if ptype not in _DTYPE:
            raise ExrError(f"channel {cname}: unknown pixel type {ptype}")
        if xs != 1 or ys != 1:
            raise ExrError(f"channel {cname}: subsampled channels are not supported")
        chans.append((cname, ptype))
    chans.sort(key=lambda c: c[0])
    comp = attrs["compression"][1][0]
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    return chans, comp, (x0, y0, x1, y1), pos


def read(path) -> Dict[str, np.ndarray]:
    """{channel: [H, W] array} of a scanline EXR file (data window)."""
    with open(path, "rb") as f:
        buf = f.read()
    chans, comp, (x0, y0, x1, y1), pos = _parse_header(buf)
    W, H = x1 - x0 + 1, y1 - y0 + 1
    if W <= 0 or H <= 0:
        raise ExrError("empty data window")
    lines = _LINES.get(comp, 1)
    nchunks = (H + lines - 1) // lines
    offsets = struct.unpack_from(f"<{nchunks}Q", buf, pos)
    out = {c: np.empty((H, W), _DTYPE[t]) for c, t in chans}
    row_bytes = [W * _DTYPE[t].itemsize for _, t in chans]
    for off in offsets:
        y, size = struct.unpack_from("<ii", buf, off)
        r0 = y - y0
        if not 0 <= r0 < H:
            raise ExrError(f"chunk at line {y} outside the data window")
        n = min(lines, H - r0)
        expected = n * sum(row_bytes)
        data = _decompress(buf[off + 8:off + 8 + size], comp, expected)
        p = 0
        for r in range(n):
            for (c, t), rb in zip(chans, row_bytes):
                out[c][r0 + r] = np.frombuffer(data, _DTYPE[t], W, p)
                p += rb
    return out


def write(path, channels: Dict[str, np.ndarray], compression: str = "ZIP") -> None:
    """Writes {channel: [H, W] array} (uint32 / float16 / float32) as a scanline EXR file."""
    comp = COMPRESSION[compression]
    if comp not in (0, 1, 2, 3):
        raise ExrError(f"writing {compression} is not supported")
    names = sorted(channels)
    arrs = []
    for c in names:
        a = np.asarray(channels[c])
        if a.dtype == np.float16:
            t = HALF
        elif a.dtype == np.float32:
            t = FLOAT
        elif a.dtype == np.uint32:
            t = UINT
        else:
            raise ExrError(f"channel {c}: dtype {a.dtype} (want uint32, float16 or float32)")
        arrs.append((c, t, np.ascontiguousarray(a, _DTYPE[t])))
    H, W = arrs[0][2].shape
    if any(a.shape != (H, W) for _, _, a in arrs):
        raise ExrError("channels differ in size")

    def attr(name, typ, payload):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(payload)) + payload

    chl = b"".join(c.encode() + b"\0" + struct.pack("<iB3xii", t, 0, 1, 1) for c, t, _ in arrs) + b"\0"
    box = struct.pack("<iiii", 0, 0, W - 1, H - 1)
    header = struct.pack("<ii", MAGIC, 2)
    header += attr("channels", "chlist", chl)
    header += attr("compression", "compression", bytes([comp]))
    header += attr("dataWindow", "box2i", box)
    header += attr("displayWindow", "box2i", box)
    header += attr("lineOrder", "lineOrder", b"\0")
    header += attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    header += attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
    header += attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    header += b"\0"
    lines = _LINES[comp]
    nchunks = (H + lines - 1) // lines
    chunks = []
    for k in range(nchunks):
        r0, r1 = k * lines, min(H, (k + 1) * lines)
        raw = b"".join(a[r].tobytes() for r in range(r0, r1) for _, _, a in arrs)
        data = _compress(raw, comp)
        if len(data) >= len(raw):
            data = raw
        chunks.append(struct.pack("<ii", r0, len(data)) + data)
    pos = len(header) + 8 * nchunks
    offsets = []
    for c in chunks:
        offsets.append(pos)
        pos += len(c)
    with open(path, "wb") as f:
        f.write(header)
        f.write(struct.pack(f"<{nchunks}Q", *offsets))
        for c in chunks:
            f.write(c)


def load(path) -> np.ndarray:
    """The image as the reference's vsg data: [H, W, 4] for R,G,B(,A); [H, W, 2]
    for two channels; [H, W] for one."""
    ch = read(path)
    names = set(ch)
    if {"R", "G", "B"} <= names:
        a = ch.get("A")
        r = ch["R"]
        return np.stack([r, ch["G"], ch["B"], a if a is not None else np.ones_like(r)], -1)
    if len(ch) == 1:
        return next(iter(ch.values()))
    if {"R", "G"} == names:
        return np.stack([ch["R"], ch["G"]], -1)
    raise ExrError(f"unsupported channel set {sorted(names)}")


def save(path, image: np.ndarray, compression: str = "ZIP") -> None:
    """Inverse of `load`: [H, W, 4] -> R,G,B,A; [H, W, 2] -> R,G; [H, W] -> R."""
    a = np.asarray(image)
    if a.ndim == 2:
        write(path, {"R": a}, compression)
    elif a.shape[-1] == 4:
        write(path, {"R": a[..., 0], "G": a[..., 1], "B": a[..., 2], "A": a[..., 3]}, compression)
    elif a.shape[-1] == 2:
        write(path, {"R": a[..., 0], "G": a[..., 1]}, compression)
    else:
        raise ExrError(f"cannot store an image of shape {a.shape}")
