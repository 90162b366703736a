#!/usr/bin/env python3
"""Regenerates the golden fixtures in tests/golden/ from the reference tree.

Run where the reference is mounted (its path is the first argument, or the
EMIDA_REFERENCE environment variable).  It converts the reference's own test fixtures to .npy, lifts
the expected offsets out of its end-to-end test, and records the outputs of the
reference's CPU code (built by `make -C oracle stage ref REF=...`) on seeded inputs, so that the
oracle stays pinned on machines where the reference tree is absent.

Sources:
  test/res/data_pic.txt, test/res/data_temp.txt       (256x256 FP64 patterns)
  test/get_offset_test.cpp:25-26, :143-193             (expected offsets)
  test/res/cross_corr/64_{A,B,res}.txt                 (integer correlation KAT)
  test/res/hann/5_{A,res}.txt, 128_{A,res}.txt         (windowed slices)
  src/subpixel_max.cpp:22-58 via oracle/_ref            (least-squares tables)
  src/cross_corr.hpp:29-65 via oracle/_ref              (serial correlation)
  src/subpixel_max.hpp:76-97 via oracle/_ref            (serial fit)
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EMIDA_REFERENCE", "")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("usage: %s REFERENCE_TREE (or set EMIDA_REFERENCE)" % sys.argv[0])


def load_matrix(path, dtype):
    """Reads the reference's square-matrix text format (src/matrix.hpp:16-27)."""
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    return np.array([float(t) for t in tok[1:1 + n * n]], dtype=np.float64).astype(dtype).reshape(n, n)


def expected_offsets():
    src = open(os.path.join(REF, "test/get_offset_test.cpp")).read()
    block = src[src.index("expected_base"):]
    block = block[:block.index("};")]
    pairs = re.findall(r"\{\s*(-?[0-9.eE+-]+)\s*,\s*(-?[0-9.eE+-]+)\s*\}", block)
    return [[float(a), float(b)] for a, b in pairs]


def main():
    out = {}
    pic = load_matrix(os.path.join(REF, "test/res/data_pic.txt"), np.float64)
    temp = load_matrix(os.path.join(REF, "test/res/data_temp.txt"), np.float64)
    np.save(os.path.join(HERE, "data_pic.npy"), pic)
    np.save(os.path.join(HERE, "data_temp.npy"), temp)

    a = load_matrix(os.path.join(REF, "test/res/cross_corr/64_A.txt"), np.int64)
    b = load_matrix(os.path.join(REF, "test/res/cross_corr/64_B.txt"), np.int64)
    r = load_matrix(os.path.join(REF, "test/res/cross_corr/64_res.txt"), np.int64)
    np.savez_compressed(os.path.join(HERE, "cross_corr_64.npz"), A=a, B=b, res=r)

    h5a = load_matrix(os.path.join(REF, "test/res/hann/5_A.txt"), np.float64)
    h5r = load_matrix(os.path.join(REF, "test/res/hann/5_res.txt"), np.float64)
    np.savez_compressed(os.path.join(HERE, "hann_5.npz"), A=h5a, res=h5r)

    # the loader fixture of test/load_tiff_test.cpp:7-49, byte for byte
    import gzip
    with open(os.path.join(REF, "test/res/INITIAL_x0y0.tif"), "rb") as src, \
            gzip.GzipFile(os.path.join(HERE, "INITIAL_x0y0.tif.gz"), "wb", 9, mtime=0) as dst:
        dst.write(src.read())

    exp = expected_offsets()
    assert len(exp) == 49, len(exp)
    out["get_offset_single"] = {"x": 0.07583538046549165, "y": -0.0982055210473689,
                                "tol": 2e-14, "source": "test/get_offset_test.cpp:25-26"}
    out["get_offset_batched"] = {"offsets": exp, "tol": 7e-13, "slice": 64, "step": 32,
                                 "cross": 127, "batch_sizes": [1, 5],
                                 "source": "test/get_offset_test.cpp:120-200"}
    with open(os.path.join(HERE, "get_offset_expected.json"), "w") as f:
        json.dump(out, f, indent=1)

    # Outputs of the reference's own CPU code on seeded inputs.
    lib_path = os.path.join(REPO, "oracle", "_ref", "libemida_ref.so")
    lib = ctypes.CDLL(lib_path)
    dp = ctypes.POINTER(ctypes.c_double)
    ref = {}
    for s in (3, 5, 7, 9):
        m = np.zeros(6 * s * s)
        assert lib.ref_lstsq_matrix(s, m.ctypes.data_as(dp)) == 0
        ref[f"lstsq_{s}"] = m
    h = np.zeros(64)
    lib.ref_hanning(ctypes.c_uint32(64), h.ctypes.data_as(dp))
    ref["hann_64"] = h
    rng = np.random.default_rng(20240607)
    for (w, hh, rw, rh, n) in ((16, 12, 31, 23, 2), (9, 9, 5, 7, 1)):
        pics = rng.normal(size=(n, hh, w))
        refs = rng.normal(size=(n, hh, w))
        res = np.zeros((n, rh, rw))
        lib.ref_cross_corr_serial(pics.ctypes.data_as(dp), refs.ctypes.data_as(dp),
                                  ctypes.c_uint32(w), ctypes.c_uint32(hh), ctypes.c_uint32(rw),
                                  ctypes.c_uint32(rh), ctypes.c_uint32(n), res.ctypes.data_as(dp))
        key = f"xcorr_{w}x{hh}_{rw}x{rh}"
        ref[key + "_pics"], ref[key + "_refs"], ref[key + "_res"] = pics, refs, res
    for s in (3, 5, 7, 9):
        n = 16
        yy, xx = np.mgrid[0:s, 0:s]
        cx = rng.uniform(s / 2 - 1, s / 2, size=n)
        cy = rng.uniform(s / 2 - 1, s / 2, size=n)
        neigh = (100 - (xx[None] - cx[:, None, None]) ** 2 * rng.uniform(1, 3, size=(n, 1, 1))
                 - (yy[None] - cy[:, None, None]) ** 2 * rng.uniform(1, 3, size=(n, 1, 1))
                 + rng.normal(scale=0.05, size=(n, s, s)))
        sub = np.zeros((n, 2))
        co = np.zeros((n, 6))
        lib.ref_subpixel_max_serial(neigh.ctypes.data_as(dp), s, ctypes.c_uint32(n),
                                    sub.ctypes.data_as(dp), co.ctypes.data_as(dp))
        ref[f"fit_{s}_neigh"], ref[f"fit_{s}_sub"], ref[f"fit_{s}_coefs"] = neigh, sub, co
    np.savez_compressed(os.path.join(HERE, "ref_cpu_outputs.npz"), **ref)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
