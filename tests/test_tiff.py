"""The command line's TIFF reader (emida_gb300/cli/tiff.hpp) on the reference's
own loader fixture, test/res/INITIAL_x0y0.tif (stored gzipped in tests/golden
by make_golden.py): an uncompressed 873 x 873 16-bit grayscale TIFF in 219
strips of 4 rows.  The reference's test (test/load_tiff_test.cpp:7-49) checks
its loader against libtiff's RGBA decoding; here the pixels are checked
against an independent parse of the IFD and its strips with numpy."""
import gzip
import os
import struct
import subprocess

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT

FIXTURE = os.path.join(GOLDEN, "INITIAL_x0y0.tif.gz")


def parse_tiff(raw):
    """Width, height and uint16 pixels from the first IFD's strips."""
    bo = "<" if raw[:2] == b"II" else ">"
    assert struct.unpack(bo + "H", raw[2:4])[0] == 42
    off = struct.unpack(bo + "I", raw[4:8])[0]
    n = struct.unpack(bo + "H", raw[off:off + 2])[0]
    tags = {}
    for i in range(n):
        e = raw[off + 2 + 12 * i:off + 14 + 12 * i]
        tag, typ, cnt = struct.unpack(bo + "HHI", e[:8])
        size = {3: 2, 4: 4}.get(typ)
        if size is None:
            continue
        fmt = bo + ("H" if size == 2 else "I") * cnt
        data = e[8:8 + size * cnt] if size * cnt <= 4 else \
            raw[struct.unpack(bo + "I", e[8:12])[0]:][:size * cnt]
        tags[tag] = struct.unpack(fmt, data)
    w, h = tags[256][0], tags[257][0]
    assert tags[258][0] == 16 and tags[259][0] == 1  # 16 bits, uncompressed
    pix = b"".join(raw[o:o + c] for o, c in zip(tags[273], tags[279]))
    return w, h, np.frombuffer(pix, dtype=bo + "u2").reshape(h, w), tags


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("tiff") / "tiff_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "tests", "tiff_driver.cpp"), "-o", exe],
                   check=True)
    return exe


def test_reader_on_the_references_fixture(driver, tmp_path):
    raw = gzip.open(FIXTURE).read()
    w, h, exp, tags = parse_tiff(raw)
    assert (w, h) == (873, 873)  # test/load_tiff_test.cpp:10
    assert len(tags[273]) == 219 and tags[278][0] == 4  # 219 strips of 4 rows
    tif = tmp_path / "INITIAL_x0y0.tif"
    tif.write_bytes(raw)
    out = tmp_path / "raster.bin"
    r = subprocess.run([driver, str(tif), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype=np.uint8)
    gw, gh = np.frombuffer(got[:8].tobytes(), dtype="<u4")
    assert (gw, gh) == (873, 873)
    pixels = np.frombuffer(got[8:].tobytes(), dtype=np.uint16).reshape(873, 873)
    assert np.array_equal(pixels, exp)
    # an EBSD pattern: the full 16-bit range is in use, not 8-bit data widened
    assert pixels.max() > 255 and (pixels >> 8).std() > 1


def test_reader_rejects_a_truncated_fixture(driver, tmp_path):
    raw = gzip.open(FIXTURE).read()
    tif = tmp_path / "cut.tif"
    tif.write_bytes(raw[:len(raw) // 2])
    r = subprocess.run([driver, str(tif), str(tmp_path / "o.bin")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and r.stderr.strip()


def test_reader_reads_only_the_requested_row_bands(driver, tmp_path):
    """load_tiff_rows, as the command line's loaders call it with the ROI row
    bands: bands that start and end inside the 4-row strips and one that
    reaches the last row; every other row is left untouched."""
    raw = gzip.open(FIXTURE).read()
    w, h, exp, _ = parse_tiff(raw)
    tif = tmp_path / "INITIAL_x0y0.tif"
    tif.write_bytes(raw)
    out = tmp_path / "rows.bin"
    bands = [(3, 10), (100, 37), (400, 1), (860, 13)]
    r = subprocess.run([driver, str(tif), str(out)] + [f"{a}:{n}" for a, n in bands],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype=np.uint8)
    pixels = np.frombuffer(got[8:].tobytes(), dtype=np.uint16).reshape(h, w)
    inside = np.zeros(h, dtype=bool)
    for a, n in bands:
        inside[a:a + n] = True
    assert np.array_equal(pixels[inside], exp[inside])
    assert (pixels[~inside] == 0xFFFF).all()
