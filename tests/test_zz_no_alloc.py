"""emida_gb_run_fft_r2c_noalloc: the forward FFT with its twiddle tables in a
fixed device array instead of allocated memory, for callers that must not
allocate device memory mid-run.  Both forms compute the same twiddles on the
host and run the same kernels, so the spectra must be the same bits, call after
call (every call rewrites the shared tables), and agree with numpy's rfft2.
The file name sorts last so the entry point is also exercised after every other
test in the same process."""
import numpy as np
import pytest

DOUBLE, FLOAT = 0, 1


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def _call(name, *args):
    from emida_gb300 import DeviceBuffer, _lib
    _lib.call(name, *[a.ptr if isinstance(a, DeviceBuffer) else a for a in args])


def _spectra(name, x, precision):
    from emida_gb300 import DeviceBuffer
    maps, h2, w2 = x.shape
    half = w2 // 2 + 1
    cdt = np.complex128 if precision == DOUBLE else np.complex64
    src = DeviceBuffer.from_array(np.ascontiguousarray(x))
    spec = DeviceBuffer(maps * h2 * half * np.dtype(cdt).itemsize)
    spec.zero()
    _call(name, src, spec, maps, w2, h2, precision)
    return spec.download(cdt, (maps, h2, half))


# consecutive calls with different sizes and precisions: each must see its own
# tables.  (1, 1024, 1024) DOUBLE fills the column table to the array's last
# byte; (2, 1024, 96) has a full-length row table beside a short column table.
CASES = [((3, 128, 128), DOUBLE), ((2, 80, 96), FLOAT), ((4, 48, 64), DOUBLE),
         ((1, 1024, 1024), FLOAT), ((1, 1024, 1024), DOUBLE), ((2, 1024, 96), DOUBLE),
         ((2, 96, 1024), FLOAT)]


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_and_numpy():
    rng = np.random.default_rng(2024)
    for (maps, h2, w2), precision in CASES:
        x = rng.normal(size=(maps, h2, w2)).astype(np.float64 if precision == DOUBLE else np.float32)
        exp = _spectra("emida_gb_run_fft_r2c", x, precision)
        got = _spectra("emida_gb_run_fft_r2c_noalloc", x, precision)
        assert np.array_equal(got, exp), ((maps, h2, w2), precision)
        ref = np.fft.rfft2(x.astype(np.float64))
        rel = 1e-12 if precision == DOUBLE else 2e-5
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err <= rel, ((maps, h2, w2), precision, err)


@pytest.mark.gpu
def test_noalloc_twice_in_a_row_same_input():
    rng = np.random.default_rng(7)
    x = rng.normal(size=(2, 64, 64))
    exp = _spectra("emida_gb_run_fft_r2c", x, DOUBLE)
    first = _spectra("emida_gb_run_fft_r2c_noalloc", x, DOUBLE)
    second = _spectra("emida_gb_run_fft_r2c_noalloc", x, DOUBLE)
    assert np.array_equal(first, exp) and np.array_equal(second, exp)


def test_noalloc_rejects_sizes_beyond_the_scratch():
    """Size checks run before any device work, so this needs no GPU."""
    from emida_gb300 import EmidaError
    for w2, h2 in [(2048, 64), (64, 1025), (0, 64)]:
        with pytest.raises(EmidaError) as ei:
            _call("emida_gb_run_fft_r2c_noalloc", None, None, 1, w2, h2, DOUBLE)
        assert ei.value.status == -1  # EMIDA_GB_INVALID_ARGUMENT
        assert "1..1024" in str(ei.value)
