"""The bounded waits of the device code: a wait on an mbarrier phase that
nothing completes runs out after its budget, the host reads the device error
word as EMIDA_GB_DEVICE_CHECK, and the context and the handle stay usable (no
fault, trap or hang is involved)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def test_wait_runs_out_and_the_handle_keeps_working():
    from emida_gb300 import EmidaError, GpuOffset, _lib, synth
    from oracle import oracle as eo
    ref = synth.reference_pattern(256, seed=61)
    pics, _ = synth.deformed_patterns(256, 61, 2, 3e-3)
    _, begins = synth.roi_grid(256, 3, 32, margin=40)
    g = GpuOffset((256, 256), begins, (64, 64), (127, 127), 2, "fft", 5, 1, "float", np.uint16, "fused")
    g.allocate_memory(ref)
    before = g.get_offset(pics)
    t0 = time.perf_counter()
    with pytest.raises(EmidaError, match="pipeline wait ran out"):
        _lib.call("emida_gb_selftest_bounded_wait", g.handle, 20_000_000)  # ~10 ms of SM clock
    assert time.perf_counter() - t0 < 30
    # the error word was read and cleared; the same handle runs the path again
    after = g.get_offset(pics)
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    o_offs, _, _ = eo.get_offsets(ref, pics, begins, 64, 64, eo.POLICY_FFT, 5)
    assert np.abs(after[0] - o_offs).max() < 1e-3
    with pytest.raises(EmidaError, match="budget"):
        _lib.call("emida_gb_selftest_bounded_wait", g.handle, 0)
    g.close()


@pytest.mark.parametrize("mode", ["fused", "plain"])
def test_failed_batch_consumes_its_ticket_and_frees_its_slot(mode):
    """A batch whose device check fails (its slot's error word set by a bounded
    wait that runs out, armed from the host) is reported by its own wait, which
    consumes the ticket; the slot then takes the next batch, whose results are
    the same as before."""
    from emida_gb300 import EmidaError, GpuOffset, _lib, synth
    ref = synth.reference_pattern(256, seed=62)
    pics, _ = synth.deformed_patterns(256, 62, 2, 3e-3)
    _, begins = synth.roi_grid(256, 3, 32, margin=40)
    g = GpuOffset((256, 256), begins, (64, 64), (127, 127), 2, "fft", 5, 1, "float", np.uint16, mode)
    g.allocate_memory(ref)
    good = g.wait(g.submit(pics))
    _lib.call("emida_gb_selftest_arm_submit", g.handle, 2_000_000)  # ~1 ms of SM clock
    bad = g.submit(pics)
    with pytest.raises(EmidaError, match="pipeline wait ran out") as ei:
        g.wait(bad)
    assert ei.value.status == -4  # EMIDA_GB_DEVICE_CHECK
    with pytest.raises(EmidaError, match="unknown ticket"):
        g.wait(bad)
    # one input buffer: the next submit reuses the failed batch's slot
    again = g.wait(g.submit(pics))
    assert np.array_equal(again[0], good[0]) and np.array_equal(again[1], good[1])
    with pytest.raises(EmidaError, match="budget"):
        _lib.call("emida_gb_selftest_arm_submit", g.handle, 0)
    g.close()
