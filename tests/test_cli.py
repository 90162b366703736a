"""The `emida` command line: the reference's flags, input files and output
lines (src/args_parser.cpp:113-283, src/process_files.hpp:235-264)."""
import os

import numpy as np
import pytest

from tests.cli_util import parse_output, run_cli, write_inputs, write_tiff


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def test_help_and_argument_errors(tmp_path):
    r = run_cli("-h")
    assert r.returncode == 0 and "--crosspolicy" in r.stderr
    r = run_cli("-i", "x.tif")
    assert r.returncode == 1 and "Argument parsing error" in r.stderr
    ref = np.zeros((128, 128), np.uint16)
    paths = write_inputs(str(tmp_path), ref, [ref], [(64, 64)], 16)
    for extra, msg in [(["--precision", "half"], "Invalid precision"),
                       (["--crosspolicy", "x"], "Invalid crosspolicy"),
                       (["-f", "4"], "fitsize 4 is not supported"),
                       (["--batchsize", "0"], "batchsize must be greater than 0"),
                       (["-c", "99,99"], "cross size must be lesser"),
                       (["--slicestep", "2,2"], "cannot use slicestep")]:
        r = run_cli("-i", paths[0], "-d", paths[1], "-b", paths[2], *extra)
        assert r.returncode == 1, extra
        assert msg in r.stderr, (extra, r.stderr)


def test_roi_out_of_bounds_and_bad_tiff(tmp_path):
    ref = np.zeros((128, 128), np.uint16)
    paths = write_inputs(str(tmp_path), ref, [ref], [(10, 64)], 16)
    r = run_cli("-i", paths[0], "-d", paths[1], "-b", paths[2])
    assert r.returncode == 1 and "out of bounds" in r.stderr
    bad = tmp_path / "bad.tif"
    bad.write_bytes(b"not a tiff")
    r = run_cli("-i", str(bad), "-d", paths[1], "-b", paths[2])
    assert r.returncode == 1


@pytest.mark.gpu
@pytest.mark.parametrize("policy,precision,fit,tol", [("fft", "double", 5, 2e-6),
                                                      ("fft", "float", 3, 2e-3),
                                                      ("brute", "double", 3, 2e-6)])
def test_cli_end_to_end_matches_oracle(tmp_path, policy, precision, fit, tol):
    from emida_gb300 import synth
    from oracle import oracle as eo
    ref = synth.reference_pattern(256, seed=41)
    pics, _ = synth.deformed_patterns(256, 41, 3, 3e-3)
    mids, begins = synth.roi_grid(256, 3, 32, margin=40)
    paths = write_inputs(str(tmp_path), ref, pics, mids, 32, big_endian=True)
    r = run_cli("-i", paths[0], "-d", paths[1], "-b", paths[2], "--precision", precision, "-f", fit,
                "--crosspolicy", policy, "--batchsize", 2, "--loadworkers", 2, "-q", "-a")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ms" in r.stderr  # -a timings
    out = parse_output(r.stdout)
    assert len(out) == 3
    pol = eo.POLICY_FFT if policy == "fft" else eo.POLICY_BRUTE
    for i, (hdr, rows) in enumerate(out):
        assert hdr[0] == 100.0 * i and hdr[1] == i * 0.5 and hdr[2] == len(mids)
        assert hdr[3].endswith(f"def_{i}.tif")
        o_offs, o_coefs, _ = eo.get_offsets(ref, pics[i:i + 1], begins, 64, 64, pol, fit)
        for k, row in enumerate(rows):
            assert (int(row[0]), int(row[1])) == tuple(mids[k])
            vals = np.array([float(v) for v in row[2:4]])
            assert np.abs(vals - o_offs[k]).max() <= tol + 1e-6
            assert len(row) == 10  # -q: six coefficients
            # "%f" keeps six decimals of each coefficient; the fit's rounding error
            # scales with the largest coefficient (the map's peak), not each one
            scale = np.abs(o_coefs[k]).max()
            rel = 1e-5 if precision == "float" else 1e-9
            assert np.abs(np.array([float(v) for v in row[4:]]) - o_coefs[k]).max() <= rel * scale + 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("mode,policy,precision", [("fused", "fft", "float"), ("tensor", "brute", "float")])
def test_cli_binary_results_match_text(tmp_path, mode, policy, precision):
    # --binary writes the same results unrounded; the text form rounds them to %f
    from emida_gb300 import read_results, synth
    ref = synth.reference_pattern(256, seed=43)
    pics, _ = synth.deformed_patterns(256, 43, 3, 3e-3)
    mids, begins = synth.roi_grid(256, 3, 32, margin=40)
    paths = write_inputs(str(tmp_path), ref, pics, mids, 32, big_endian=False)
    common = ["-i", paths[0], "-d", paths[1], "-b", paths[2], "--precision", precision, "-f", 5,
              "--crosspolicy", policy, "--batchsize", 2, "--mode", mode]
    text = run_cli(*common, "-q")
    assert text.returncode == 0, text.stdout + text.stderr
    out = tmp_path / "results.bin"
    r = run_cli(*common, "--binary", out)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == ""  # the results went to the file
    got = read_results(out)
    expect = parse_output(text.stdout)
    assert len(got) == len(expect) == 3
    for g, (hdr, rows) in zip(got, expect):
        assert (g["x"], g["y"], len(g["mids"]), g["name"]) == (hdr[0], hdr[1], hdr[2], hdr[3])
        vals = np.array([[float(v) for v in row] for row in rows])
        assert np.array_equal(g["mids"], vals[:, :2].astype(np.uint32))
        assert np.abs(g["offsets"] - vals[:, 2:4]).max() <= 5e-7
        assert np.abs(g["coefs"] - vals[:, 4:]).max() <= 5e-7 * max(1.0, np.abs(g["coefs"]).max())
