"""Helpers for driving the `emida` command line in tests: an independent
uncompressed 16-bit TIFF writer (several strips, either byte order) and the
reference's input-file formats (src/args_parser.cpp:67-111,
src/process_files.hpp:56-75)."""
import os
import struct
import subprocess

import numpy as np

from tests.conftest import ROOT

CLI = os.path.join(ROOT, "emida_gb300", "bin", "emida")


def write_tiff(path, img, rows_per_strip=4, big_endian=False):
    img = np.ascontiguousarray(img, dtype=np.uint16)
    h, w = img.shape
    e = ">" if big_endian else "<"
    data = img.astype(e + "u2").tobytes()
    strips = [data[r * w * 2:min(h, r + rows_per_strip) * w * 2] for r in range(0, h, rows_per_strip)]
    n = len(strips)
    entries = 10
    ifd = 8
    after_ifd = ifd + 2 + 12 * entries + 4
    offs_at = after_ifd
    counts_at = offs_at + 4 * n
    data_at = counts_at + 4 * n
    offsets, pos = [], data_at
    for s in strips:
        offsets.append(pos)
        pos += len(s)

    def ent(tag, typ, count, value):
        if typ == 3 and count == 1:
            return struct.pack(e + "HHIHH", tag, typ, count, value, 0)
        return struct.pack(e + "HHII", tag, typ, count, value)

    out = (b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, ifd)
    out += struct.pack(e + "H", entries)
    out += ent(256, 4, 1, w) + ent(257, 4, 1, h) + ent(258, 3, 1, 16) + ent(259, 3, 1, 1)
    out += ent(262, 3, 1, 1) + ent(273, 4, n, offs_at if n > 1 else offsets[0])
    out += ent(274, 3, 1, 1) + ent(277, 3, 1, 1) + ent(278, 4, 1, rows_per_strip)
    out += ent(279, 4, n, counts_at if n > 1 else len(strips[0]))
    out += struct.pack(e + "I", 0)
    if n > 1:
        out += struct.pack(e + f"{n}I", *offsets) + struct.pack(e + f"{n}I", *[len(s) for s in strips])
    else:
        out += b"\0" * (8 * n)
    out += b"".join(strips)
    with open(path, "wb") as f:
        f.write(out)


def write_inputs(tmp, ref, pics, mids, radius, big_endian=False):
    write_tiff(os.path.join(tmp, "ref.tif"), ref)
    with open(os.path.join(tmp, "def.txt"), "w") as f:
        for i, p in enumerate(pics):
            name = os.path.join(tmp, f"def_{i}.tif")
            write_tiff(name, p, rows_per_strip=7, big_endian=big_endian and i % 2 == 1)
            f.write(f"{100.0 * i} {i * 0.5} {name}\n")
    with open(os.path.join(tmp, "roi.txt"), "w") as f:
        f.write(f"{radius}\n")
        for x, y in mids:
            f.write(f"{int(x)} {int(y)}\n")
    return [os.path.join(tmp, n) for n in ("ref.tif", "def.txt", "roi.txt")]


def run_cli(*args, timeout=300):
    return subprocess.run([CLI, *map(str, args)], capture_output=True, text=True, timeout=timeout)


def parse_output(text, coefs=False):
    """[(header fields, [(mid_x, mid_y, dx, dy[, 6 coefs])...])] per pattern."""
    lines = text.strip().splitlines()
    out, i = [], 0
    while i < len(lines):
        x, y, n, name = lines[i].split(" ", 3)
        rows = [lines[i + 1 + k].split() for k in range(int(n))]
        out.append(((float(x), float(y), int(n), name), rows))
        i += 1 + int(n)
    return out
