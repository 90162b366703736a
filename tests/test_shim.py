"""The C++ shim (include/emida_gb/gpu_offset.hpp): a caller written against the
reference's interface (src/gpu_offset.hpp:48-326, src/get_offset.hpp:7-20),
compiled and linked against libemida_gb.so, gives the results of the library's
own API and the reference's golden single pair, and fails with
std::runtime_error where the reference's CUCH would throw."""
import json
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT

EXPECTED = json.load(open(os.path.join(GOLDEN, "get_offset_expected.json")))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    import __graft_entry__
    __graft_entry__.build_library()
    exe = str(tmp_path_factory.mktemp("shim") / "shim_driver")
    lib_dir = os.path.join(ROOT, "emida_gb300")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    # the driver uses its own CUDA runtime beside the library's, as the
    # reference's callers do (cudaMallocHost, cudaMemcpy, cudaStreamSynchronize)
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "shim_driver.cpp"), "-L", lib_dir, "-lemida_gb",
                    "-L", os.path.join(cuda, "lib64"), "-lcudart",
                    f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", exe],
                   check=True)
    return exe


def test_shim_compiles_and_throws_runtime_error(driver):
    r = subprocess.run([driver, "validate"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "runtime_error: Wrong fitting size" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("policy,precision,mode", [(1, 1, 2), (1, 0, 1), (0, 0, 1), (0, 1, 3)])
def test_shim_pipeline_equals_library_api(driver, tmp_path, policy, precision, mode):
    # FFT float fused; FFT double plain; brute double plain; brute float tensor
    from emida_gb300 import GpuOffset, synth
    w, batch, s = 384, 3, 5
    ref = synth.reference_pattern(w, seed=51)
    pics, _ = synth.deformed_patterns(w, 51, batch, 3e-3)
    _, begins = synth.roi_grid(w, 3, 32, margin=48)
    n = len(begins)
    src = tmp_path / "in.bin"
    with open(src, "wb") as f:
        f.write(np.array([w, w, n, batch, policy, precision, s, mode], np.uint32).tobytes())
        f.write(np.asarray(begins, np.uint32).tobytes())
        f.write(np.ascontiguousarray(ref, np.uint16).tobytes())
        f.write(np.ascontiguousarray(pics, np.uint16).tobytes())
    dst = tmp_path / "out.bin"
    r = subprocess.run([driver, "run", str(src), str(dst)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(dst, np.float64)
    N = batch * n
    one_o, one_c = raw[:2 * N].reshape(N, 2), raw[2 * N:8 * N].reshape(N, 6)
    two_o, two_c = raw[8 * N:10 * N].reshape(N, 2), raw[10 * N:].reshape(N, 6)
    names = {0: "plain", 1: "plain", 2: "fused", 3: "tensor"}
    g = GpuOffset((w, w), begins, (64, 64), (127, 127), batch, "fft" if policy else "brute", s, 1,
                  "float" if precision else "double", np.uint16, names[mode])
    g.allocate_memory(ref)
    offs, coefs = g.get_offset(pics)
    g.close()
    assert np.array_equal(one_o, offs) and np.array_equal(one_c, coefs)
    # get_offset_core + finalize fits on the host in the reference's operation order
    assert np.array_equal(two_o, offs) and np.array_equal(two_c, coefs)


@pytest.mark.gpu
def test_shim_free_get_offset_golden_pair(driver, tmp_path):
    # test/get_offset_test.cpp:10-27 through the free function get_offset<double>
    pic = np.load(os.path.join(GOLDEN, "data_pic.npy"))[:64, :64]
    temp = np.load(os.path.join(GOLDEN, "data_temp.npy"))[:64, :64]
    src = tmp_path / "pair.bin"
    with open(src, "wb") as f:
        f.write(np.array([64], np.uint32).tobytes())
        f.write(np.ascontiguousarray(pic, np.float64).tobytes())
        f.write(np.ascontiguousarray(temp, np.float64).tobytes())
    dst = tmp_path / "pair_out.bin"
    r = subprocess.run([driver, "pair", str(src), str(dst)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    x, y = np.fromfile(dst, np.float64)
    e = EXPECTED["get_offset_single"]
    assert abs(x - e["x"]) <= e["tol"] and abs(y - e["y"]) <= e["tol"]


@pytest.mark.gpu
@pytest.mark.parametrize("policy,precision,mode", [(1, 1, 0), (1, 0, 1), (0, 0, 1)])
def test_shim_process_files_sequence(driver, tmp_path, policy, precision, mode):
    """The call sequence of the reference's file_processor
    (src/process_files.hpp:98-233): three load workers calling
    transfer_pic_to_device_async from pinned rasters, a compute thread that
    synchronises offs.in_stream before get_offset_core, a finalize thread.
    11 patterns in batches of 4 (the last one short): each result equals the
    library's own get_offset of that batch."""
    from emida_gb300 import GpuOffset, synth
    w, batch, s, n_pat, workers = 384, 4, 5, 11, 3
    ref = synth.reference_pattern(w, seed=52)
    pics, _ = synth.deformed_patterns(w, 52, n_pat, 3e-3)
    _, begins = synth.roi_grid(w, 3, 32, margin=48)
    n = len(begins)
    src = tmp_path / "files.bin"
    with open(src, "wb") as f:
        f.write(np.array([w, w, n, batch, policy, precision, s, mode, n_pat, workers], np.uint32).tobytes())
        f.write(np.asarray(begins, np.uint32).tobytes())
        f.write(np.ascontiguousarray(ref, np.uint16).tobytes())
        f.write(np.ascontiguousarray(pics, np.uint16).tobytes())
    dst = tmp_path / "files_out.bin"
    r = subprocess.run([driver, "files", str(src), str(dst)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(dst, np.float64)
    N = n_pat * n
    got_o, got_c = raw[:2 * N].reshape(N, 2), raw[2 * N:].reshape(N, 6)
    names = {0: "auto", 1: "plain"}
    g = GpuOffset((w, w), begins, (64, 64), (127, 127), batch, "fft" if policy else "brute", s, 1,
                  "float" if precision else "double", np.uint16, names[mode])
    g.allocate_memory(ref)
    for c in range(0, n_pat, batch):
        part = np.zeros((batch, w, w), np.uint16)
        part[:min(batch, n_pat - c)] = pics[c:c + batch]
        offs, coefs = g.get_offset(part)
        k = min(batch, n_pat - c) * n
        assert np.array_equal(got_o[c * n:c * n + k], offs[:k]), c
        assert np.array_equal(got_c[c * n:c * n + k], coefs[:k]), c
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1])
def test_shim_cross_corr_fft_hooks(driver, tmp_path, mode):
    """test/cross_corr_fft_test.cpp:8-46 through the shim's get_cu_pic(),
    get_cu_temp() and cross_corr_fft(), for the form AUTO picks (fused, whose
    hook buffers are made on first use) and the staged form: the correlation
    map is the unnormalised inverse of rfft2(pic) times the conjugate of the
    spectrum written into get_cu_temp()."""
    dst = tmp_path / f"hooks{mode}.bin"
    r = subprocess.run([driver, "hooks", str(mode), str(dst)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(dst, np.float64).reshape(8, 8)
    a = np.array([[1, 2, 3, 1], [4, 5, 6, 1], [7, 8, 9, 1], [7, 8, 9, 1]], np.float64)
    b = np.array([[6, 3, 2, 1], [12, 23, 3, 1], [1, 8, 9, 1], [7, 8, 9, 1]], np.float64)
    pic = np.zeros((8, 8))
    pic[:4, :4] = a
    temp_real = np.zeros((8, 10))
    temp_real[:4, :4] = b
    temp = temp_real[:, 0::2] + 1j * temp_real[:, 1::2]  # [8][5] complex, as the buffer is read
    exp = np.fft.irfft2(np.fft.rfft2(pic) * np.conj(temp), s=(8, 8)) * 64
    assert np.abs(got - exp).max() <= 1e-12 * np.abs(exp).max()
