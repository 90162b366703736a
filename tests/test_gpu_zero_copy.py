"""Patterns in pinned host memory read in place by the kernels (zero-copy):
every entry that accepts them gives the same bits as the copied or
device-resident run of the same patterns."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


@pytest.fixture(scope="module")
def data():
    from emida_gb300 import synth
    ref = synth.reference_pattern(512, seed=41)
    pics, _ = synth.deformed_patterns(512, 41, 6, sigma_eps=3e-3)
    _, begins = synth.roi_grid(512, 4, 32, margin=48)
    return ref, pics, begins


@pytest.mark.parametrize("policy,mode", [("fft", "fused"), ("brute", "tensor"), ("fft", "plain")])
def test_run_device_on_pinned_host_patterns(data, policy, mode):
    from emida_gb300 import DeviceBuffer, GpuOffset, _lib, pinned_array
    ref, pics, begins = data
    n, S = len(pics), len(begins)
    g = GpuOffset((512, 512), begins, (64, 64), (127, 127), n, policy, 5, 1, "float", np.uint16, mode)
    g.allocate_memory(ref)
    host = pinned_array(pics.shape)
    host[:] = pics
    d_pics = DeviceBuffer.from_array(pics)
    o_dev, o_host = DeviceBuffer(n * S * 16), DeviceBuffer(n * S * 16)
    g.run_device(d_pics, n, o_dev)
    g.run_device(host.ctypes.data, n, o_host)
    _lib.call("emida_gb_synchronize")
    assert np.array_equal(o_dev.download(np.float64, (n * S, 2)), o_host.download(np.float64, (n * S, 2)))
    g.close()


def test_pageable_patterns_are_refused_by_run_device(data):
    from emida_gb300 import DeviceBuffer, EmidaError, GpuOffset
    ref, pics, begins = data
    g = GpuOffset((512, 512), begins, (64, 64), (127, 127), 2, "fft", 5, 1, "float", np.uint16, "fused")
    g.allocate_memory(ref)
    pageable = np.ascontiguousarray(pics[:2])
    with pytest.raises(EmidaError, match="pinned host memory"):
        g.run_device(pageable.ctypes.data, 2, DeviceBuffer(2 * len(begins) * 16))
    g.close()


def test_submit_reads_pinned_batches_in_place(data):
    from emida_gb300 import GpuOffset, pinned_array
    ref, pics, begins = data
    g = GpuOffset((512, 512), begins, (64, 64), (127, 127), 3, "fft", 5, 3, "float", np.uint16, "fused")
    g.allocate_memory(ref)
    assert g.ingest == "sm_copy"  # the default of the fused form (1024-byte rows)
    host = pinned_array(pics.shape)
    host[:] = pics
    expect = [g.get_offset(pics[k:k + 3]) for k in (0, 3)]
    for mode in ("in_place", "copy", "sm_copy"):
        g.ingest = mode
        assert g.ingest == mode  # 16 ROIs of 64^2 cover a quarter of a 512^2 pattern
        tickets = [g.submit(host[k:k + 3]) for k in (0, 3, 0)]
        for t, (e_offs, e_coefs) in zip(tickets, expect + expect[:1]):
            offs, coefs = g.wait(t)
            assert np.array_equal(offs, e_offs) and np.array_equal(coefs, e_coefs)
    g.close()
    # ROIs that cover most of the pattern are copied, not read in place
    _, dense = __import__("emida_gb300").synth.roi_grid(512, 7, 32, margin=32)
    g = GpuOffset((512, 512), dense, (64, 64), (127, 127), 1, "fft", 5, 1, "float", np.uint16, "fused")
    g.ingest = "in_place"
    assert g.ingest == "copy"
    g.close()


def test_multi_run_table_mixes_device_and_host_patterns(data):
    from emida_gb300 import DeviceBuffer, MultiLayout, pinned_array, synth
    ref, pics, begins = data
    m = MultiLayout((512, 512), "float")
    lay = [(begins, 64, 5)]
    for r, s, n in ((24, 3, 7), (48, 9, 3), (64, 5, 2)):  # 96-, 192-point fused, 256 staged
        _, b = synth.random_layout(512, 60 + r, r, n, margin=4)
        lay.append((b, 2 * r, s))
    for b, side, s in lay:
        m.add_layout(b, side, s, ref)
    layout_of = np.array([0, 1, 2, 3, 1, 0], dtype=np.uint32)
    total = m.count(layout_of)
    d_pics = DeviceBuffer.from_array(pics)
    o_arr, o_tab = DeviceBuffer(total * 16), DeviceBuffer(total * 16)
    m.run(d_pics, layout_of, o_arr, graph=False)
    host = pinned_array(pics.shape)
    host[:] = pics
    ptrs = [host[p] if p % 2 else d_pics.ptr.value + p * 512 * 512 * 2 for p in range(len(pics))]
    m.run_table(ptrs, layout_of, o_tab)
    m.synchronize()
    expect = o_arr.download(np.float64, (total, 2))
    assert np.array_equal(expect, o_tab.download(np.float64, (total, 2)))
    # a pattern that does not start on a 16-byte boundary: the table is staged
    # with plain loads instead of 16-byte chunks, with the same bits
    flat = pinned_array((pics.size + 8,))
    odd = flat[1:1 + pics.size].reshape(pics.shape)
    odd[:] = pics
    o_odd = DeviceBuffer(total * 16)
    m.run_table([odd[p] if p == 2 else host[p] for p in range(len(pics))], layout_of, o_odd)
    m.synchronize()
    assert np.array_equal(expect, o_odd.download(np.float64, (total, 2)))
    m.close()


def test_server_rows_in_place_equal_copied_rows(data):
    from emida_gb300 import Server, pinned_array, synth
    ref, pics, begins = data
    # `wide` covers most of the pattern: copied under "sparse", read in place by default
    _, wide = synth.roi_grid(512, 7, 32, margin=32)
    results = {}
    for zero_copy in (False, "sparse", True):
        s = Server("float", hbm_bytes=8 * 512 * 512 * 2, step_patterns=4, zero_copy=zero_copy)
        sparse = s.add_layout((512, 512), begins, 64, 5, ref)
        dense = s.add_layout((512, 512), wide, 64, 3, ref)
        rows = []
        for k in range(4):
            host = pinned_array((3, 512, 512))
            host[:] = pics[k:k + 3]
            rows.append((sparse if k % 2 == 0 else dense, host))
        rids = [s.submit(lid, h) for lid, h in rows]
        results[zero_copy] = [s.wait(r)[:2] for r in rids]
        s.close()
    for level in ("sparse", True):
        for (a_offs, a_coefs), (b_offs, b_coefs) in zip(results[False], results[level]):
            assert np.array_equal(a_offs, b_offs) and np.array_equal(a_coefs, b_coefs)


def _ragged_begins(w, h, side, n, seed):
    # x at every remainder mod 8, the right and bottom edges included
    rng = np.random.default_rng(seed)
    xs = list(rng.integers(0, w - side + 1, n - 2)) + [w - side, 0]
    ys = list(rng.integers(0, h - side + 1, n - 2)) + [h - side, h - side]
    return np.array(list(zip(xs, ys)), dtype=np.int64)


@pytest.mark.parametrize("side,precision,mode", [(32, "float", "fused"), (24, "float", "fused"),
                                                 (48, "float", "fused"), (96, "float", "fused"),
                                                 (128, "float", "fused"), (32, "double", "fused"),
                                                 (64, "float", "tensor")])
def test_submit_gather_ingest_equals_copy(side, precision, mode):
    # the gather kernel packs only the ROI rows of a pinned batch; the path then
    # reads the compact layout and gives the bits of the copied batch
    from emida_gb300 import GpuOffset, pinned_array, synth
    w, h, batch = 520, 384, 3
    ref = synth.reference_pattern((w, h), seed=side)
    pics, _ = synth.deformed_patterns((w, h), side, 2 * batch, sigma_eps=3e-3)
    # the compact layout (ROIs of side x ((side + 14) & ~7) pixels) fits in a pattern
    begins = _ragged_begins(w, h, side, 8 if side == 128 else 12, seed=side)
    assert {int(x) % 8 for x, _ in begins} != {0}
    policy = "brute" if mode == "tensor" else "fft"
    g = GpuOffset((w, h), begins, (side, side), (2 * side - 1, 2 * side - 1), batch, policy, 5, 3,
                  precision, np.uint16, mode)
    g.allocate_memory(ref)
    host = pinned_array(pics.shape)
    host[:] = pics
    expect = [g.get_offset(pics[k:k + batch]) for k in (0, batch)]
    g.ingest = "gather"
    assert g.ingest == "gather"
    tickets = [g.submit(host[k:k + batch]) for k in (0, batch, 0)]
    for t, (e_offs, e_coefs) in zip(tickets, expect + expect[:1]):
        offs, coefs = g.wait(t)
        assert np.array_equal(offs, e_offs) and np.array_equal(coefs, e_coefs)
    # a partial batch, and a batch that is not 16-byte aligned (copied instead)
    t = g.submit(host[:2])
    offs, _ = g.wait(t)
    assert np.array_equal(offs, expect[0][0][:2 * len(begins)])
    flat = pinned_array((batch * w * h + 8,))
    odd = flat[1:1 + batch * w * h].reshape(batch, h, w)
    odd[:] = pics[:batch]
    offs, coefs = g.wait(g.submit(odd))
    assert np.array_equal(offs, expect[0][0]) and np.array_equal(coefs, expect[0][1])
    g.close()


def test_gather_ingest_needs_its_geometry():
    from emida_gb300 import GpuOffset, synth
    ref = synth.reference_pattern((260, 256), seed=3)
    # a width that is not a multiple of 8
    g = GpuOffset((260, 256), [(0, 0), (100, 90)], (64, 64), (127, 127), 1, "fft", 5, 1, "float",
                  np.uint16, "fused")
    assert g.ingest == "copy"  # the default where the SM copy is not allowed
    g.ingest = "gather"
    assert g.ingest == "copy"
    # nor are its 520-byte rows whole 16-byte chunks for the SM copy
    g.ingest = "sm_copy"
    assert g.ingest == "copy"
    g.close()
    # a compact layout larger than the pattern (overlapping ROIs)
    many = [(k % 190, k % 190) for k in range(40)]
    g = GpuOffset((256, 256), many, (64, 64), (127, 127), 1, "fft", 5, 1, "float", np.uint16, "fused")
    g.ingest = "gather"
    assert g.ingest == "copy"
    g.close()
    # the staged form and FP64 input read whole patterns
    for mode, in_type in (("plain", np.uint16), ("fused", np.float64)):
        g = GpuOffset((256, 256), [(0, 0)], (64, 64), (127, 127), 1, "fft", 5, 1, "float", in_type, mode)
        # the staged form leaves no CTA slots for the SM copy: the copy engine is its default
        assert g.ingest == ("copy" if mode == "plain" else "sm_copy")
        g.ingest = "gather"
        assert g.ingest == "copy"
        g.close()


@pytest.mark.parametrize("side,precision,mode,in_type,n_rois", [
    (32, "float", "fused", np.uint16, 12), (48, "float", "fused", np.uint16, 3),
    (64, "float", "tensor", np.uint16, 12), (32, "float", "plain", np.uint16, 12),
    (32, "double", "fused", np.float64, 12), (32, "float", "fused", np.uint16, 60)])
def test_submit_sm_copy_ingest_equals_copy(side, precision, mode, in_type, n_rois):
    # the row bands of a pinned batch copied by SM loads instead of the copy
    # engine: the bits of the copied batch, for sparse bands, a single band and
    # bands that cover the whole pattern (60 ROIs)
    from emida_gb300 import GpuOffset, pinned_array, synth
    w, h, batch = 520, 384, 3
    ref = synth.reference_pattern((w, h), seed=side + 1)
    pics, _ = synth.deformed_patterns((w, h), side + 1, 2 * batch, sigma_eps=3e-3)
    pics = pics.astype(in_type)
    begins = _ragged_begins(w, h, side, n_rois, seed=side + n_rois)
    policy = "brute" if mode == "tensor" else "fft"
    g = GpuOffset((w, h), begins, (side, side), (2 * side - 1, 2 * side - 1), batch, policy, 5, 3,
                  precision, in_type, mode)
    g.allocate_memory(ref.astype(in_type))
    host = pinned_array(pics.shape, in_type)
    host[:] = pics
    expect = [g.get_offset(pics[k:k + batch]) for k in (0, batch)]
    g.ingest = "sm_copy"
    assert g.ingest == "sm_copy"
    tickets = [g.submit(host[k:k + batch]) for k in (0, batch, 0)]
    for t, (e_offs, e_coefs) in zip(tickets, expect + expect[:1]):
        offs, coefs = g.wait(t)
        assert np.array_equal(offs, e_offs) and np.array_equal(coefs, e_coefs)
    # a partial batch, and a batch that is not 16-byte aligned (copied instead)
    offs, _ = g.wait(g.submit(host[:2]))
    assert np.array_equal(offs, expect[0][0][:2 * len(begins)])
    flat = pinned_array((batch * w * h + 8,), in_type)
    odd = flat[1:1 + batch * w * h].reshape(batch, h, w)
    odd[:] = pics[:batch]
    offs, coefs = g.wait(g.submit(odd))
    assert np.array_equal(offs, expect[0][0]) and np.array_equal(coefs, expect[0][1])
    g.close()
