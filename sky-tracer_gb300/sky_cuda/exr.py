"""Minimal OpenEXR and PNG files for the output stage (no third-party codec).

write_exr_rgb   single-part scanline OpenEXR, channels B/G/R as 32-bit float,
                no compression (the reference writes its band and RGB images
                as float RGB EXRs through the `exr` crate, film_output.rs:84-109)
read_exr        scanline OpenEXR with NONE, RLE, ZIPS or ZIP compression and
                HALF / FLOAT / UINT channels (what --rebuild-rgb-only reads back,
                film_output.rs:136-156); returns {channel: [H, W] array}
write_png_rgb8  8-bit RGB PNG, filter 0, zlib (film_output.rs:111-134)

Layouts follow the public OpenEXR file-format document and the PNG
specification.
"""

from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

EXR_MAGIC = 20000630
NO_COMPRESSION, RLE_COMPRESSION, ZIPS_COMPRESSION, ZIP_COMPRESSION = 0, 1, 2, 3
_PIXEL_TYPES = {0: np.dtype("<u4"), 1: np.dtype("<f2"), 2: np.dtype("<f4")}
_LINES_PER_BLOCK = {NO_COMPRESSION: 1, RLE_COMPRESSION: 1, ZIPS_COMPRESSION: 1, ZIP_COMPRESSION: 16}


class ExrError(ValueError):
    pass


def _attr(name: str, kind: str, payload: bytes) -> bytes:
    return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<i", len(payload)) + payload


def write_exr_rgb(path, rgb: np.ndarray) -> None:
    """Write [H, W, 3] float values as an uncompressed scanline float RGB EXR."""
    rgb = np.asarray(rgb, dtype="<f4")
    if rgb.ndim != 3 or rgb.shape[2] != 3:
        raise ExrError("expected an [H, W, 3] array")
    h, w = rgb.shape[:2]
    channels = b"".join(c.encode() + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1) for c in ("B", "G", "R")) + b"\0"
    header = b"".join([
        _attr("channels", "chlist", channels),
        _attr("compression", "compression", bytes([NO_COMPRESSION])),
        _attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)),
        _attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)),
        _attr("lineOrder", "lineOrder", bytes([0])),
        _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)),
        _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)),
        _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)),
    ]) + b"\0"
    prefix = struct.pack("<ii", EXR_MAGIC, 2) + header
    line_bytes = 3 * w * 4
    chunk = 8 + line_bytes
    first = len(prefix) + 8 * h
    offsets = struct.pack(f"<{h}Q", *[first + y * chunk for y in range(h)])
    body = bytearray()
    for y in range(h):
        body += struct.pack("<ii", y, line_bytes)
        for c in (2, 1, 0):  # channel order B, G, R (sorted by name)
            body += rgb[y, :, c].tobytes()
    Path(path).write_bytes(prefix + offsets + bytes(body))


def _read_header(buf: bytes):
    if len(buf) < 8 or struct.unpack_from("<i", buf, 0)[0] != EXR_MAGIC:
        raise ExrError("not an OpenEXR file")
    version = struct.unpack_from("<i", buf, 4)[0]
    if version & 0x200 or version & 0x800 or version & 0x1000:
        raise ExrError("tiled, deep or multi-part EXR files are not supported")
    pos, attrs = 8, {}
    while buf[pos] != 0:
        end = buf.index(b"\0", pos)
        name = buf[pos:end].decode()
        pos = end + 1
        end = buf.index(b"\0", pos)
        kind = buf[pos:end].decode()
        pos = end + 1
        size = struct.unpack_from("<i", buf, pos)[0]
        pos += 4
        attrs[name] = (kind, buf[pos:pos + size])
        pos += size
    return attrs, pos + 1


def _parse_channels(payload: bytes):
    out, pos = [], 0
    while payload[pos] != 0:
        end = payload.index(b"\0", pos)
        name = payload[pos:end].decode()
        ptype, _linear, xs, ys = struct.unpack_from("<iB3xii", payload, end + 1)
        if xs != 1 or ys != 1:
            raise ExrError("subsampled channels are not supported")
        out.append((name, ptype))
        pos = end + 1 + 16
    return out


def _unpredict(data: bytes) -> bytes:
    """Undo the EXR ZIP/RLE byte predictor and the even/odd split."""
    t = np.frombuffer(data, dtype=np.uint8).astype(np.int32)
    t = ((np.cumsum(t - 128, dtype=np.int64) + 128) % 256).astype(np.uint8)
    half = (len(t) + 1) // 2
    out = np.empty(len(t), dtype=np.uint8)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def _rle_decode(data: bytes, expected: int) -> bytes:
    out, i = bytearray(), 0
    while i < len(data) and len(out) < expected:
        count = struct.unpack_from("b", data, i)[0]
        i += 1
        if count < 0:
            out += data[i:i - count]
            i -= count
        else:
            out += bytes([data[i]]) * (count + 1)
            i += 1
    return bytes(out)


def read_exr(path) -> dict:
    """{channel name: [H, W] float32 array} of a scanline EXR file."""
    buf = Path(path).read_bytes()
    attrs, pos = _read_header(buf)
    try:
        channels = _parse_channels(attrs["channels"][1])
        compression = attrs["compression"][1][0]
        x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    except KeyError as e:
        raise ExrError(f"missing EXR attribute {e}") from e
    if compression not in _LINES_PER_BLOCK:
        raise ExrError(f"EXR compression {compression} is not supported (NONE, RLE, ZIPS, ZIP are)")
    w, h = x1 - x0 + 1, y1 - y0 + 1
    per = _LINES_PER_BLOCK[compression]
    blocks = (h + per - 1) // per
    offsets = struct.unpack_from(f"<{blocks}Q", buf, pos)
    sizes = [_PIXEL_TYPES[t].itemsize for _, t in channels]
    out = {name: np.zeros((h, w), dtype=np.float32) for name, _ in channels}
    for off in offsets:
        y, size = struct.unpack_from("<ii", buf, off)
        data = buf[off + 8:off + 8 + size]
        lines = min(per, y1 + 1 - y)
        raw_len = lines * w * sum(sizes)
        if compression in (ZIPS_COMPRESSION, ZIP_COMPRESSION) and size < raw_len:
            data = _unpredict(zlib.decompress(data))
        elif compression == RLE_COMPRESSION and size < raw_len:
            data = _unpredict(_rle_decode(data, raw_len))
        p = 0
        for line in range(lines):
            for (name, ptype), sz in zip(channels, sizes):
                row = np.frombuffer(data, dtype=_PIXEL_TYPES[ptype], count=w, offset=p)
                out[name][y - y0 + line] = row.astype(np.float32)
                p += w * sz
    return out


def write_png_rgb8(path, rgb8: np.ndarray) -> None:
    """Write an [H, W, 3] uint8 image as an RGB PNG."""
    rgb8 = np.ascontiguousarray(rgb8, dtype=np.uint8)
    h, w = rgb8.shape[:2]

    def chunk(kind: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xffffffff)

    raw = b"".join(b"\0" + rgb8[y].tobytes() for y in range(h))
    png = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
           chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
    Path(path).write_bytes(png)


def read_png_rgb8(path) -> np.ndarray:
    """[H, W, 3] uint8 of an 8-bit RGB, non-interlaced PNG written with filter 0."""
    buf = Path(path).read_bytes()
    if buf[:8] != b"\x89PNG\r\n\x1a\n":
        raise ExrError("not a PNG file")
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(buf):
        length = struct.unpack_from(">I", buf, pos)[0]
        kind = buf[pos + 4:pos + 8]
        data = buf[pos + 8:pos + 8 + length]
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack_from(">IIBB", data)
            if depth != 8 or ctype != 2:
                raise ExrError("only 8-bit RGB PNGs are read")
        elif kind == b"IDAT":
            idat += data
        pos += 12 + length
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + 3 * w)
    if np.any(raw[:, 0] != 0):
        raise ExrError("only PNG filter type 0 is read")
    return raw[:, 1:].reshape(h, w, 3).copy()
