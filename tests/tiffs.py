"""A writer of baseline TIFF files for the TIFF-folder tests: the layouts the
reader must decode (both byte orders, several strips, SHORT or LONG fields,
chunky and planar multi-sample pixels, fields it must skip) and the ones it
must refuse (16-bit, compressed, tiled).  Written from the TIFF 6.0 field
layout: an 8-byte header, image data, then one image directory of 12-byte
entries sorted by tag."""
from __future__ import annotations

import struct

import numpy as np

BYTE, ASCII, SHORT, LONG, RATIONAL = 1, 2, 3, 4, 5
_SIZE = {BYTE: 1, ASCII: 1, SHORT: 2, LONG: 4, RATIONAL: 8}
_FMT = {BYTE: "B", ASCII: "B", SHORT: "H", LONG: "I", RATIONAL: "II"}


def tiff_bytes(img: np.ndarray, big_endian=False, rows_per_strip=None, planar=1, long_fields=False,
               bits=8, compression=1, tiled=False, extra_fields=True, omit_counts=False) -> bytes:
    """img: [h, w] or [h, w, samples] uint8 (uint16 when bits=16)."""
    e = ">" if big_endian else "<"
    if img.ndim == 2:
        img = img[:, :, None]
    h, w, spp = img.shape
    rps = h if rows_per_strip is None else rows_per_strip
    dt = np.dtype(e + ("u1" if bits == 8 else "u2"))
    strips = []
    if planar == 1:
        for y0 in range(0, h, rps):
            strips.append(np.ascontiguousarray(img[y0:y0 + rps]).astype(dt).tobytes())
    else:
        for s in range(spp):
            for y0 in range(0, h, rps):
                strips.append(np.ascontiguousarray(img[y0:y0 + rps, :, s]).astype(dt).tobytes())
    out = bytearray(b"MM" if big_endian else b"II")
    out += struct.pack(e + "HI", 42, 0)
    offsets = []
    for sb in strips:
        offsets.append(len(out))
        out += sb
        if len(out) % 2:
            out += b"\0"
    desc = b"synthetic slice\0"
    fields = {}
    ilong = LONG if long_fields else SHORT
    fields[256] = (ilong, [w])
    fields[257] = (ilong, [h])
    fields[258] = (SHORT, [bits] * spp)
    fields[259] = (SHORT, [compression])
    fields[262] = (SHORT, [1])
    if extra_fields:
        fields[270] = (ASCII, list(desc))
    fields[273] = (LONG, offsets)
    fields[277] = (SHORT, [spp])
    fields[278] = (ilong, [rps])
    if not omit_counts:
        fields[279] = (LONG, [len(sb) for sb in strips])
    if extra_fields:
        fields[282] = (RATIONAL, [72, 1])
        fields[283] = (RATIONAL, [72, 1])
    if spp > 1:
        fields[284] = (SHORT, [planar])
    if tiled:
        fields[322] = (SHORT, [16])
        fields[323] = (SHORT, [16])
    fields[339] = (SHORT, [1] * spp)
    # Values that do not fit in 4 bytes go before the directory.
    placed = {}
    for tag, (typ, vals) in sorted(fields.items()):
        n = len(vals) // (2 if typ == RATIONAL else 1)
        if n * _SIZE[typ] > 4:
            if len(out) % 2:
                out += b"\0"
            placed[tag] = len(out)
            out += struct.pack(e + _FMT[typ][0] * len(vals), *vals)
    if len(out) % 2:
        out += b"\0"
    ifd = len(out)
    struct.pack_into(e + "I", out, 4, ifd)
    out += struct.pack(e + "H", len(fields))
    for tag, (typ, vals) in sorted(fields.items()):
        n = len(vals) // (2 if typ == RATIONAL else 1)
        if tag in placed:
            out += struct.pack(e + "HHII", tag, typ, n, placed[tag])
        else:
            raw = struct.pack(e + _FMT[typ][0] * len(vals), *vals).ljust(4, b"\0")
            out += struct.pack(e + "HHI", tag, typ, n) + raw
    out += struct.pack(e + "I", 0)
    return bytes(out)


def write_folder(folder, volume: np.ndarray, name="slice_{:04d}.tif", **kw):
    """volume [z, y, x] (or [z, y, x, samples]) as one file per z slice."""
    import os
    os.makedirs(folder, exist_ok=True)
    for z in range(volume.shape[0]):
        with open(os.path.join(folder, name.format(z)), "wb") as f:
            f.write(tiff_bytes(volume[z], **kw))
