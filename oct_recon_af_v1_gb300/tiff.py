"""Legacy TIFF output on the GB300 kernels (octrecon/io/tiff_writer.py:53-71).

`write_legacy_tiff` keeps the reference's signature and file: a BigTIFF with
one page per output y plane (nZ rows x nX columns, uint16 codes), PackBits
compression, the "Software" tag of the first page holding the JSON
{"metadata", "clim", "version": 3}, and the same JSON in `<path>.json`.  The
codes (db_to_bits, optionally the legacy double quantisation) and the
PackBits packets are computed on the device; this module only lays out the
file.  No tifffile / imagecodecs is needed.

`read_legacy_tiff` reads such a file back (codes and metadata): the
counterpart of the reference's loader for checking a written volume.
"""
from __future__ import annotations

import json
import struct
from pathlib import Path

import numpy as np

from ._lib import Context

_SHORT, _LONG, _ASCII, _LONG8 = 3, 4, 2, 16
_SIZE = {_SHORT: 2, _LONG: 4, _ASCII: 1, _LONG8: 8}


def _entry(tag, typ, values):
    """(tag, type, count, payload bytes) of one IFD entry."""
    if typ == _ASCII:
        payload = values.encode("ascii") + b"\0"
        return tag, typ, len(payload), payload
    fmt = {_SHORT: "<H", _LONG: "<I", _LONG8: "<Q"}[typ]
    values = list(values) if isinstance(values, (list, tuple, np.ndarray)) else [values]
    return tag, typ, len(values), b"".join(struct.pack(fmt, int(v)) for v in values)


def _write_ifd(f, entries):
    """Write an IFD at the current position (payloads > 8 bytes just before it);
    returns (ifd offset, offset of its next-IFD field)."""
    blobs = {}
    for tag, typ, count, payload in entries:
        if len(payload) > 8:
            if f.tell() % 2:
                f.write(b"\0")
            blobs[tag] = f.tell()
            f.write(payload)
    if f.tell() % 2:
        f.write(b"\0")
    ifd = f.tell()
    f.write(struct.pack("<Q", len(entries)))
    for tag, typ, count, payload in sorted(entries):
        f.write(struct.pack("<HHQ", tag, typ, count))
        f.write(struct.pack("<Q", blobs[tag]) if tag in blobs else payload.ljust(8, b"\0"))
    nxt = f.tell()
    f.write(struct.pack("<Q", 0))
    return ifd, nxt


def write_legacy_tiff(path, db_volume, clim, metadata: dict, legacy_double_quantization: bool = False,
                      plane_clims=None, progress=None, device: int = 0, rows_per_strip: int | None = None):
    """db_volume: (nY, nZ, nX) float32 — numpy array / memmap, or a CUDA tensor."""
    path = Path(path)
    meta = {"metadata": metadata, "clim": [float(clim[0]), float(clim[1])], "version": 3}
    meta_json = json.dumps(meta, separators=(",", ":"))
    c1, c2 = sorted(float(v) for v in clim)
    ny, nz, nx = db_volume.shape
    rps = rows_per_strip or max(1, 65536 // (2 * nx))
    ctx = Context(device)
    try:
        with open(path, "wb") as f:
            f.write(b"II" + struct.pack("<HHHQ", 43, 8, 0, 0))
            prev_next = 8                                    # the header's first-IFD field
            for yi in range(ny):
                plane = db_volume[yi]
                if not hasattr(plane, "data_ptr"):
                    plane = np.ascontiguousarray(plane, dtype=np.float32)
                if legacy_double_quantization:
                    pc = plane_clims[yi] if plane_clims is not None else ctx.minmax(plane)
                    bits = ctx.quantise_double(plane, pc, (c1, c2))
                else:
                    bits = ctx.quantise(plane, (c1, c2))
                data, sizes = ctx.packbits(bits)
                row_off = np.concatenate([[0], np.cumsum(sizes, dtype=np.int64)])
                strip_off, strip_cnt = [], []
                base = f.tell()
                f.write(data)
                for r0 in range(0, nz, rps):
                    r1 = min(nz, r0 + rps)
                    strip_off.append(base + int(row_off[r0]))
                    strip_cnt.append(int(row_off[r1] - row_off[r0]))
                entries = [_entry(256, _LONG, nx), _entry(257, _LONG, nz), _entry(258, _SHORT, 16),
                           _entry(259, _SHORT, 32773), _entry(262, _SHORT, 1), _entry(273, _LONG8, strip_off),
                           _entry(277, _SHORT, 1), _entry(278, _LONG, rps), _entry(279, _LONG8, strip_cnt),
                           _entry(339, _SHORT, 1)]
                if yi == 0:
                    entries.append(_entry(305, _ASCII, meta_json))
                ifd, nxt = _write_ifd(f, entries)
                end = f.tell()
                f.seek(prev_next)
                f.write(struct.pack("<Q", ifd))
                f.seek(end)
                prev_next = nxt
                if progress:
                    progress(yi)
    finally:
        ctx.close()
    with open(path.with_suffix(path.suffix + ".json"), "w") as f:
        json.dump(meta, f)


def packbits_decode(buf: bytes) -> bytes:
    """TIFF PackBits decoding (compression 32773)."""
    out = bytearray()
    i, n = 0, len(buf)
    while i < n:
        h = buf[i]
        i += 1
        if h < 128:
            out += buf[i:i + h + 1]
            i += h + 1
        elif h > 128:
            out += bytes([buf[i]]) * (257 - h)
            i += 1
    return bytes(out)


def read_legacy_tiff(path):
    """-> (codes (nY, nZ, nX) uint16, metadata dict or None) of a file written
    by write_legacy_tiff (BigTIFF, PackBits or uncompressed uint16 pages)."""
    data = Path(path).read_bytes()
    if data[:4] != b"II+\0":
        raise ValueError("not a little-endian BigTIFF")
    off = struct.unpack_from("<Q", data, 8)[0]
    pages, meta = [], None
    while off:
        n = struct.unpack_from("<Q", data, off)[0]
        tags = {}
        for k in range(n):
            tag, typ, count = struct.unpack_from("<HHQ", data, off + 8 + 20 * k)
            raw = data[off + 8 + 20 * k + 12: off + 8 + 20 * k + 20]
            size = _SIZE[typ] * count
            payload = raw[:size] if size <= 8 else data[struct.unpack("<Q", raw)[0]:][:size]
            if typ == _ASCII:
                tags[tag] = payload.rstrip(b"\0").decode("ascii")
            else:
                fmt = {_SHORT: "H", _LONG: "I", _LONG8: "Q"}[typ]
                tags[tag] = list(struct.unpack("<" + fmt * count, payload))
        nx, nz = tags[256][0], tags[257][0]
        comp = tags.get(259, [1])[0]
        raw_rows = b"".join(packbits_decode(data[o:o + c]) if comp == 32773 else data[o:o + c]
                            for o, c in zip(tags[273], tags[279]))
        pages.append(np.frombuffer(raw_rows, "<u2").reshape(nz, nx))
        if 305 in tags and meta is None:
            meta = json.loads(tags[305])
        off = struct.unpack_from("<Q", data, off + 8 + 20 * n)[0]
    return np.stack(pages), meta
