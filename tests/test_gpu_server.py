"""The request loop: rows of different pattern sizes and layouts submitted
concurrently share steps on the device; each row's result equals the row run
alone, and rows wait for arena room (admission by free HBM)."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


@pytest.fixture(scope="module")
def world():
    from emida_gb300 import synth
    sizes = {512: synth.reference_pattern(512, seed=31), 256: synth.reference_pattern(256, seed=32)}
    # (pattern size, ROI side, fit size, ROI count): native and zero-padded sides
    specs = [(512, 64, 5, 9), (512, 50, 3, 6), (512, 76, 7, 4), (256, 48, 9, 5), (256, 40, 5, 4)]
    layouts = []
    for i, (w, side, s, n) in enumerate(specs):
        _, begins = synth.random_layout(w, 200 + i, side // 2, n, margin=4)
        layouts.append((w, begins, side, s))
    rng = np.random.default_rng(5)
    rows = []
    for k in range(14):
        lid = int(rng.integers(0, len(layouts)))
        w = layouts[lid][0]
        n = int(rng.integers(2, 9))
        pics, _ = synth.deformed_patterns(w, 31 if w == 512 else 32, n, 3e-3, first=5 * k)
        rows.append((lid, pics))
    return sizes, layouts, rows


def make_server(sizes, layouts, budget_patterns=16, step=6, precision="float"):
    from emida_gb300 import Server
    s = Server(precision, hbm_bytes=budget_patterns * 512 * 512 * 2, step_patterns=step)
    for w, begins, side, fs in layouts:
        s.add_layout((w, w), begins, side, fs, sizes[w])
    return s


def test_rows_alone_equal_rows_mixed(world):
    sizes, layouts, rows = world
    alone = []
    s = make_server(sizes, layouts)
    for lid, pics in rows:
        alone.append(s.wait(s.submit(lid, pics))[:2])
    s.close()
    # all rows at once from four threads with jitter; budget forces waiting
    s = make_server(sizes, layouts, budget_patterns=16, step=6)
    results = {}
    lock = threading.Lock()

    def client(idx):
        for k in idx:
            time.sleep(0.002 * (k % 3))
            rid = s.submit(*rows[k])
            with lock:
                results[k] = rid

    threads = [threading.Thread(target=client, args=(list(range(t, len(rows), 4)),)) for t in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k in range(len(rows)):
        offs, coefs, lat = s.wait(results[k])
        assert lat > 0
        assert np.array_equal(offs, alone[k][0]) and np.array_equal(coefs, alone[k][1])
    st = s.stats()
    assert st["completed"] == len(rows) and 0 < st["p50_ms"] <= st["p99_ms"]
    assert st["pairs_per_s"] > 0
    s.close()


def test_server_rows_match_oracle(world):
    from oracle import oracle as eo
    from tests.test_gpu_synthetic import well_posed
    sizes, layouts, rows = world
    s = make_server(sizes, layouts)
    for lid, pics in rows[:4]:
        w, begins, side, fs = layouts[lid]
        offs, coefs, _ = s.wait(s.submit(lid, pics))
        o_offs, o_coefs, _ = eo.get_offsets(sizes[w], pics, begins, side, side, eo.POLICY_FFT, fs)
        ok = well_posed(o_coefs, fs)
        assert (np.abs(offs - o_offs).max(axis=1)[ok] <= 1e-3).all()
    s.close()


def test_row_larger_than_arena_is_refused(world):
    from emida_gb300 import EmidaError
    sizes, layouts, rows = world
    s = make_server(sizes, layouts, budget_patterns=4)
    lid = next(i for i, l in enumerate(layouts) if l[0] == 512)
    big = np.zeros((5, 512, 512), dtype=np.uint16)
    with pytest.raises(EmidaError, match="exceeds"):
        s.submit(lid, big)
    s.close()


def test_long_copied_row_equals_its_patterns_alone(world):
    # a copied row longer than the copy window (8 chunks of 16 patterns): its
    # copies are queued over many rounds of the loop while steps of it run
    from emida_gb300 import Server, synth
    sizes, layouts, _ = world
    lid = next(i for i, l in enumerate(layouts) if l[0] == 256)
    w, begins, side, fs = layouts[lid]
    pics, _ = synth.deformed_patterns(256, 32, 30, 3e-3, first=200)
    long_row = np.ascontiguousarray(np.tile(pics, (10, 1, 1)))  # 300 pageable patterns: copied
    s = Server("float", hbm_bytes=512 * 256 * 256 * 2, step_patterns=64)
    ids = [s.add_layout((l[0], l[0]), l[1], l[2], l[3], sizes[l[0]]) for l in layouts]
    alone_offs, alone_coefs, _ = s.wait(s.submit(ids[lid], pics))
    offs, coefs, _ = s.wait(s.submit(ids[lid], long_row))
    n = len(begins)
    assert offs.shape == (300 * n, 2)
    for k in range(10):
        sl = slice(30 * n * k, 30 * n * (k + 1))
        assert np.array_equal(offs[sl], alone_offs) and np.array_equal(coefs[sl], alone_coefs)
    s.close()


def test_trace_records_every_row_in_order_of_its_stages(world):
    """emida_gb_server_trace: one record per completed row with its pattern
    count, and times from submission that do not decrease from admission to
    first step launch, last step launch and completion."""
    sizes, layouts, rows = world
    s = make_server(sizes, layouts, budget_patterns=16, step=6)
    ids = [s.submit(lid, pics) for lid, pics in rows]
    for rid in ids:
        s.wait(rid)
    tr = s.trace()
    s.close()
    assert tr.shape == (len(rows), 5)
    assert sorted(tr[:, 0].astype(int).tolist()) == sorted(len(p) for _, p in rows)
    assert (tr[:, 1] >= 0).all()
    assert (np.diff(tr[:, 1:], axis=1) >= 0).all()
