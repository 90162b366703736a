#!/usr/bin/env python3
"""Throughput of the ROI cross-correlation path: ROI pairs/s.

Workload (the detector-size configuration): 256 deformed synthetic EBSD
patterns of 1024 x 1024 uint16 against one reference pattern, 100 ROIs of
64 x 64 (radius 32) on a 10 x 10 grid (margin 40), FFT policy (128 x 128
transforms), fit size 5, batch size 32.  One step is the whole 256-pattern job.
Synthetic data: 32 distinct seeded deformed patterns repeated to 256 (every
pair is computed; the 512 MB pattern set is larger than the 129 MB L2, so no
L2 flush is needed between steps).

value: device-resident throughput of the chosen form (inputs in HBM when the
timed region starts), CUDA events on the launching stream.
e2e: the same job through the public C ABI (submit/wait) from pinned host
memory, three batches in flight: per batch the host->device copy (overlapping
the previous batch's path; only the row bands that hold ROI pixels are
copied), the path, and the offsets, coefficients and maxima back to the host.
The timed steps run as one stream of batches, as a scan is processed;
one_step_ms is a single step with the pipeline filled and drained inside it.
e2e_ingest: the same with the other ingest modes (kernels reading each batch's
ROI pixels in place, gathered ROI rows, row bands copied by the copy engine).
plain_reference: the reference's own staged GPU pipeline (its gpu_offset with
cuFFT, compiled from its sources for sm_103a) on the same job, device-resident
and end to end; over_plain_reference gives this form's ratios to it.
fp64, tensor, serving: the job in float64 (fused form beside the reference's
float64 pipeline), the brute policy on the tensor cores at fit size 7, and
rows of the detector layout arriving at 100 rows/s for 4 s (p50/p99).

cpu_baseline and --impl reference time the reference's own CPU code on all host
cores (sums_serial, cross_corr_serial over the 127 x 127 lags -- it has no CPU
FFT path -- and subpixel_max_serial, compiled from its sources staged into
baseline/_ref), in the GPU arm's precision, on a bounded sample of the job's
pairs; cpu_port_fft is the oracle's FP64 FFT restatement beside it.

Multi-GPU: patterns are independent, so N ranks each process their own 256
patterns (weak scaling, no collective on the data path).
"""
import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from emida_gb300.shard import dist_env, max_over_ranks, whole_job_rate  # noqa: E402

METRIC = "ROI pairs/s at <=0.01 px vs FP64 oracle"
UNIQUE = 32
# DRAM traffic of the fused FP32 kernel on this workload, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum) of a 12,800-pair launch: 177.9 MB,
# of which 6.66 MB are the once-per-launch reference spectra; scaled by pairs.
TRAFFIC_PER_PAIR = (177.9e6 - 6.66e6) / 12800
TRAFFIC_PER_LAUNCH = 6.66e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="float", choices=["float", "double"])
    ap.add_argument("--mode", default="fused", choices=["fused", "plain"])
    ap.add_argument("--patterns", type=int, default=256)
    ap.add_argument("--profile-case", type=int, default=0,
                    help="run only N patterns through the chosen form a few times (for ncu)")
    ap.add_argument("--profile-target", default="fused",
                    choices=["fused", "cluster", "homography", "ingest", "inplace", "fused64",
                             "fused96", "fused192"],
                    help="profile case: the detector's fused kernel; the 256-point cluster kernel "
                         "(1024^2, 6 x 6 ROIs of 128^2); the deformation fit (N patterns x 100 ROIs); "
                         "N detector patterns from pinned host memory through submit/wait, copied "
                         "and then gathered, three batches of 32 in flight; the fused kernel reading N "
                         "pinned host detector patterns in place (cp.async staging); the 64-, 96- "
                         "and 192-point fused kernels (1024^2, 10 x 10 ROIs of 32^2, 48^2 or 96^2)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form comparison")
    ap.add_argument("--no-legs", action="store_true",
                    help="skip the reference's staged GPU pipeline, the FP64, tensor and serving legs")
    ap.add_argument("--sample-seconds", type=float, default=0.0,
                    help="reference arm: seconds of host work per step (default: ~20 s in all)")
    ap.add_argument("--in-flight", type=int, default=3,
                    help="e2e: batches in flight through submit/wait (device input buffers)")
    ap.add_argument("--config", default="detector",
                    choices=["detector", "batching", "serving", "precision", "cli"],
                    help="detector: 256 x 1024^2, 100 ROIs r=32 (default); batching: patterns on "
                         "uneven layouts; serving: Poisson stream of scan rows; precision: 2048 "
                         "patterns, brute on the tensor cores beside the FP32 FFT; cli: the emida "
                         "command line from TIFF files to text")
    ap.add_argument("--rate", type=float, default=50.0, help="serving: rows per second")
    ap.add_argument("--duration", type=float, default=8.0, help="serving: seconds of arrivals")
    ap.add_argument("--layout", default="mixed", choices=["mixed", "detector"],
                    help="serving: mixed sizes and layouts, or the detector grid at 1024^2")
    ap.add_argument("--step-patterns", type=int, default=128, help="serving: patterns per step")
    ap.add_argument("--in-place-rows", action="store_true",
                    help="serving: the kernels read every pinned row in place (no copy into the arena)")
    return ap.parse_args()


def workload(seed=2024):
    from emida_gb300 import synth
    ref = synth.reference_pattern(1024, seed)
    uniq, _ = synth.deformed_patterns(1024, seed, UNIQUE, sigma_eps=5e-3)
    mids, begins = synth.roi_grid(1024, 10, 32, margin=40)
    return ref, uniq, begins


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region (the body
    of the `with`): samples every 20 ms, read with their arrival times by a
    thread; the region starts only once the first sample has arrived, and only
    samples that arrive inside it (or the first one after it, for a region
    shorter than the sampling interval) are summarised."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.stamped = []
        self.lines = []

    def _read(self):
        for line in self.proc.stdout:
            if line.strip():
                self.stamped.append((time.perf_counter(), line.strip()))

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        if self.proc:
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
            deadline = time.perf_counter() + 5.0
            while not self.stamped and time.perf_counter() < deadline and self.proc.poll() is None:
                time.sleep(0.005)
        self.t0 = time.perf_counter()
        return self

    def __exit__(self, *exc):
        t1 = time.perf_counter()
        if self.proc:
            time.sleep(0.05)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()
            self.reader.join(timeout=5)
            inside = [l for t, l in self.stamped if self.t0 <= t <= t1]
            after = [l for t, l in self.stamped if t > t1]
            self.lines = inside or after[:1]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[2:6]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def well_posed(coefs, s):
    """Fits whose extremum lies inside the s x s window (elsewhere the offset is
    an extrapolation of a nearly flat quadratic)."""
    b, c, d, e, f = (coefs[:, k] for k in range(1, 6))
    y = (b * e - 2 * c * d) / (4 * f * d - e * e)
    x = (-e * y - b) / (2 * d)
    return np.repeat(((x >= 0) & (x <= s - 1) & (y >= 0) & (y <= s - 1))[:, None], 2, axis=1)


DETECTOR_WORKLOAD = "256 x 1024^2 uint16 patterns, 100 ROIs r=32 (64x64), FFT 128x128, s=5, batch 32"


def detector_config(P, S, world, precision):
    """The detector workload's config object, the same in both arms."""
    return {"workload": DETECTOR_WORKLOAD, "patterns": P, "rois": S, "radius": 32, "fitsize": 5,
            "batch": 32, "precision": precision, "l2": "inputs larger than L2 (512 MB of patterns)",
            "parallelism": f"patterns sharded over {world} GPU(s)"}


def cpu_port(ref, uniq, begins, seconds, threads):
    """The oracle's C restatement (FP64, FFT policy, s=5) on the host cores:
    (pairs/s, pairs, seconds)."""
    from oracle import oracle as eo
    eo.lib()
    stop = time.perf_counter() + seconds
    counts = []
    lock = threading.Lock()

    def worker(k):
        n = 0
        i = k
        while time.perf_counter() < stop:
            eo.get_offsets(ref, uniq[i % len(uniq)][None], begins, 64, 64, eo.POLICY_FFT, 5)
            n += len(begins)
            i += threads
        with lock:
            counts.append(n)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(worker, range(threads)))
    dt = time.perf_counter() - t0
    pairs = sum(counts)
    return pairs / dt, pairs, dt


class CpuReference:
    """The reference's own CPU code on the host cores, one ROI pair per call:
    sums_serial, generate_hanning, cross_corr_serial (127 x 127 lags; the
    reference has no CPU FFT path) and subpixel_max_serial, in `precision`,
    compiled from its sources into oracle/_ref (oracle/ref_harness.cpp).
    Falls back to the oracle port where oracle/_ref was not built."""

    def __init__(self, ref, uniq, begins, precision):
        from oracle import oracle as eo
        self.eo, self.uniq, self.begins, self.precision = eo, uniq, begins, precision
        self.ref, self.lib = ref, eo.ref_lib()
        self.kind = "reference" if self.lib is not None else "port"
        if self.lib is not None:
            self.prep = eo.ref_prepare_reference(self.lib, ref, begins, 64, precision)

    def pair(self, i):
        S = len(self.begins)
        p, r = (i // S) % len(self.uniq), i % S
        return self.eo.ref_brute_pattern(self.lib, self.prep[r:r + 1], self.uniq[p], self.begins[r:r + 1],
                                         64, 127, 5, self.precision)

    def parity(self, n_pairs):
        """Max |offset - FP64 oracle| (px) and peak agreement over the first pairs."""
        eo = self.eo
        o_offs, _, o_peaks = eo.get_offsets(self.ref, self.uniq[:1], self.begins, 64, 64,
                                            eo.POLICY_BRUTE, 5, 127, 127)
        got = [self.pair(i) for i in range(n_pairs)]
        err = max(float(np.abs(o[0] - o_offs[i]).max()) for i, o in enumerate(got))
        match = float(np.mean([o[1][0] == o_peaks[i] for i, o in enumerate(got)]))
        return err, match

    def run(self, seconds, threads):
        """(pairs/s, pairs, seconds) of `seconds` of work on `threads` threads."""
        if self.lib is None:
            return cpu_port(self.ref, self.uniq, self.begins, seconds, threads)
        stop = time.perf_counter() + seconds
        counter = iter(range(1 << 40))
        lock = threading.Lock()
        done = []

        def worker(_):
            n = 0
            while time.perf_counter() < stop:
                with lock:
                    i = next(counter)
                self.pair(i)
                n += 1
            with lock:
                done.append(n)

        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(worker, range(threads)))
        dt = time.perf_counter() - t0
        return sum(done) / dt, sum(done), dt


def run_reference(args, rank, world):
    """The reference's own CPU implementation of the path on all host cores,
    on the detector workload's pairs, in the GPU arm's precision; each step is
    a bounded sample of that workload."""
    if rank != 0:
        return
    ref, uniq, begins = workload()
    threads = os.cpu_count() or 1
    per_step = args.sample_seconds or max(0.5, 20.0 / max(1, args.steps + args.warmup))
    cpu = CpuReference(ref, uniq, begins, args.precision)
    err, match = cpu.parity(2) if cpu.kind == "reference" else (None, None)
    vals = []
    for i in range(args.warmup + args.steps):
        v, pairs, dt = cpu.run(per_step, threads)
        if i >= args.warmup:
            vals.append((v, pairs, dt))
    value = sum(p for _, p, _ in vals) / sum(d for _, _, d in vals)
    what = (f"the reference's own CPU code (sums_serial, cross_corr_serial over 127x127 lags, "
            f"subpixel_max_serial) in {args.precision}, one ROI pair per call on {threads} threads"
            if cpu.kind == "reference" else "the oracle's FP64 C restatement (FFT policy)")
    sample = (f"{sum(p for _, p, _ in vals)} ROI pairs of the workload over {args.steps} steps of "
              f"~{per_step:.1f} s: {what}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "ROI pairs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * 25600 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision == "float" else "f64", "data": "synthetic",
        "config": detector_config(256, len(begins), world, args.precision),
        "cpu_baseline": {"value": value, "unit": "ROI pairs/s", "cores": threads, "kind": cpu.kind,
                         "sample": sample},
        "parity": {"max_abs_err_px": err, "peak_match_rate": match,
                   "vs": "FP64 oracle (brute), first 2 pairs"},
        "e2e": {"value": value, "unit": "ROI pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


INGEST_HOW = {
    "copy": "one pitched copy-engine copy per row band",
    "sm_copy": "each row band by SM loads on 16 CTAs beside the previous batch's path",
}


def roi_rows(begins, side):
    """Pattern rows that hold ROI pixels (the rows a batch copy moves)."""
    rows = np.zeros(1 + max(int(y) for _, y in begins) + side, dtype=bool)
    for _, y in begins:
        rows[int(y):int(y) + side] = True
    return int(rows.sum())


def pinned_u16(shape):
    """A uint16 array in pinned host memory (freed with the process)."""
    import ctypes
    from emida_gb300 import _lib
    n = int(np.prod(shape))
    p = ctypes.c_void_p()
    _lib.call("emida_gb_malloc_host", ctypes.byref(p), n * 2)
    return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint16)), (n,)).reshape(shape)


def random_layouts(size, count, seed, radii, rois, margin=4):
    """`count` seeded layouts: (begins, side, fit size)."""
    from emida_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        r = int(rng.choice(radii)) if len(radii) > 2 else int(rng.integers(radii[0], radii[1] + 1))
        n = int(rng.integers(rois[0], rois[1] + 1))
        _, begins = synth.random_layout(size, seed * 100 + i, r, n, margin=margin)
        out.append((begins, 2 * r, int(rng.choice([3, 5, 7, 9]))))
    return out


def run_batching(args):
    """4096 patterns of 1024^2 on 32 seeded layouts (radius 16..64, 25-400 ROIs,
    fit size 3..9): one multi-layout run per step, replayed from a CUDA graph,
    grids autotuned per ROI size."""
    import __graft_entry__
    __graft_entry__.build_library()
    print(json.dumps(batching_measure(args.precision, args.steps, args.warmup)), flush=True)


def batching_measure(precision, steps, warmup):
    """The batching workload of run_batching; returns its JSON object."""
    import time
    from emida_gb300 import DeviceBuffer, MultiLayout, _lib, synth
    from oracle import oracle as eo
    P, L = 4096, 32
    ref = synth.reference_pattern(1024, 77)
    uniq, _ = synth.deformed_patterns(1024, 77, L, sigma_eps=5e-3)
    layouts = random_layouts(1024, L, 77, [16, 24, 32, 48, 64], (25, 400))
    m = MultiLayout((1024, 1024), precision)
    for begins, side, fs in layouts:
        m.add_layout(begins, side, fs, ref)
    layout_of = np.arange(P, dtype=np.uint32) % L
    d_pics = DeviceBuffer(P * 1024 * 1024 * 2)
    d_uniq = DeviceBuffer.from_array(uniq)
    import ctypes
    for k in range(P // L):  # the 32 patterns repeated, on the device
        _lib.call("emida_gb_memcpy_d2d", ctypes.c_void_p(d_pics.ptr.value + k * L * 1024 * 1024 * 2),
                  d_uniq.ptr, L * 1024 * 1024 * 2)
    total = m.count(layout_of)
    d_offs, d_coefs = DeviceBuffer(total * 16), DeviceBuffer(total * 48)
    report = m.autotune(d_pics, layout_of, d_offs)
    d_maxes = DeviceBuffer(total * m.data_index.itemsize)
    m.run(d_pics, layout_of, d_offs, d_coefs, d_maxes, graph=True)
    m.synchronize()
    # parity: the first pattern of every layout against the FP64 oracle
    offs = d_offs.download(np.float64, (total, 2))
    coefs = d_coefs.download(np.float64, (total, 6))
    peaks = d_maxes.download(m.data_index, total)["index"]
    import concurrent.futures as cf
    starts = np.concatenate([[0], np.cumsum([len(layouts[l][0]) for l in layout_of])])

    def check(p):
        begins, side, fs = layouts[layout_of[p]]
        o, c, pk = eo.get_offsets(ref, uniq[p:p + 1], begins, side, side, eo.POLICY_FFT, fs)
        sl = slice(starts[p], starts[p + 1])
        ok = well_posed(c, fs)
        d = np.abs(offs[sl] - o)[ok]
        return (float(d.max()) if d.size else 0.0, int(ok.sum() // 2), len(o), float((d ** 2).sum()),
                d.size, int((peaks[sl] == pk).sum()))
    with cf.ThreadPoolExecutor(os.cpu_count()) as ex:
        res = list(ex.map(check, range(L)))
    err = max(r[0] for r in res)
    rms = float(np.sqrt(sum(r[3] for r in res) / max(1, sum(r[4] for r in res))))
    peak_match = sum(r[5] for r in res) / sum(r[2] for r in res)
    assert err <= 1e-2, f"offset error {err} px"
    for _ in range(warmup):
        m.run(d_pics, layout_of, d_offs, d_coefs, graph=True)
    m.synchronize()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(steps):
            m.run(d_pics, layout_of, d_offs, d_coefs, graph=True)
        m.synchronize()
        dt = (time.perf_counter() - t0) / steps
    radii = sorted({l[1] // 2 for l in layouts})
    out = {
        "metric": "ROI pairs/s, patterns on uneven ROI layouts (one graph-replayed multi-layout run)",
        "value": total / dt, "unit": "ROI pairs/s", "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": dt * 1000, "higher_is_better": True,
        "dtype": "f32" if precision == "float" else "f64", "data": "synthetic",
        "config": {"workload": f"{P} x 1024^2 uint16 patterns on {L} seeded layouts, radius "
                               f"{radii}, 25-400 ROIs, fit 3-9", "patterns": P, "pairs": int(total)},
        "autotune": report.strip().splitlines(),
        "parity": {"max_abs_err_px": err, "rms_err_px": rms, "peak_match_rate": peak_match,
                   "well_posed_fits": sum(r[1] for r in res), "checked_pairs": sum(r[2] for r in res),
                   "vs": "FP64 oracle, one pattern per layout"},
        "clocks": clk.summary()}
    m.close()
    return out


def run_serving(args):
    """A Poisson stream of scan rows of 32-512 patterns through the request
    loop; p50/p99 row latency and sustained ROI pairs/s.  --layout mixed:
    512^2 or 1024^2 rows (50/50), each on one of 8 seeded layouts per size
    (25-225 ROIs of radius 24-48, fit 3-9).  --layout detector: 1024^2 rows on
    the 10 x 10 grid of 64 x 64 ROIs, fit 5."""
    import __graft_entry__
    __graft_entry__.build_library()
    print(json.dumps(serving_measure(args.precision, args.layout, args.rate, args.duration,
                                     args.step_patterns, args.in_place_rows)), flush=True)


def serving_measure(precision, layout, rate, duration, step_patterns, in_place):
    """The serving workload of run_serving; returns its JSON object."""
    from emida_gb300 import Server, synth
    from oracle import oracle as eo
    rng = np.random.default_rng(99)
    detector = layout == "detector"
    sizes = (1024,) if detector else (512, 1024)
    srv = Server(precision, hbm_bytes=24 << 30, step_patterns=step_patterns,
                 zero_copy=bool(in_place))
    rows_src, layouts = {}, {}
    for size in sizes:
        ref = synth.reference_pattern(size, 90 + size)
        uniq, _ = synth.deformed_patterns(size, 90 + size, 16, sigma_eps=5e-3)
        buf = pinned_u16((512, size, size))
        for i in range(512):
            buf[i] = uniq[i % 16]
        rows_src[size] = (ref, buf)
        if detector:
            _, grid = synth.roi_grid(size, 10, 32, margin=40)
            lay = [(grid, 64, 5)] * 8
        else:
            lay = random_layouts(size, 8, size, (24, 48), (25, 225))
        layouts[size] = [(srv.add_layout((size, size), b, side, fs, ref), b, side, fs) for b, side, fs in lay]
    # parity of one row per size against the FP64 oracle (not timed)
    errs, sq = [], []
    for size in sizes:
        lid, begins, side, fs = layouts[size][0]
        ref, buf = rows_src[size]
        offs, coefs, _ = srv.wait(srv.submit(lid, buf[:2]))
        o, c, _ = eo.get_offsets(ref, buf[:2], begins, side, side, eo.POLICY_FFT, fs)
        ok = well_posed(c, fs)
        d = np.abs(offs - o)[ok]
        errs.append(float(d.max()))
        sq.append(d ** 2)
    # every layout once before the stream (not timed), as a deployment does
    # when it registers its layouts
    for size in sizes:
        for lid, *_ in layouts[size]:
            srv.wait(srv.submit(lid, rows_src[size][1][:2]))
    srv.reset_stats()
    # arrivals
    pending, sent_pairs = [], 0
    t_end = time.perf_counter() + duration
    with ClockSampler(0) as clk:
        t = time.perf_counter()
        while t < t_end:
            size = 1024 if detector or rng.random() >= 0.5 else 512
            lid, begins, side, fs = layouts[size][int(rng.integers(0, 8))]
            n = int(rng.integers(32, 513))
            pending.append(srv.submit(lid, rows_src[size][1][:n]))
            sent_pairs += n * len(begins)
            t += rng.exponential(1.0 / rate)
            delay = t - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
        for rid in pending:
            srv.wait(rid)
    st = srv.stats()
    tr = srv.trace()
    srv.close()
    # where the slowest 1 % of rows spent their time: queued before admission,
    # waiting for their first step, between first and last step, and from the
    # last step's launch to completion
    slow = tr[np.argsort(tr[:, 4])[-max(1, len(tr) // 100):]] if len(tr) else tr
    tail = [{"patterns": int(r[0]), "admit_ms": r[1], "first_launch_ms": r[2], "last_launch_ms": r[3],
             "done_ms": r[4]} for r in slow]
    return {
        "metric": "row latency p50/p99 and ROI pairs/s under a Poisson stream of scan rows",
        "value": st["pairs_per_s"], "unit": "ROI pairs/s", "n_gpus": 1,
        "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"]}, "rows": st["completed"],
        "slowest_rows": tail,
        "pairs": sent_pairs, "higher_is_better": True,
        "dtype": "f32" if precision == "float" else "f64", "data": "synthetic",
        "config": {"workload": ("Poisson rows: 32-512 patterns of 1024^2, 100 ROIs of 64x64 (10x10 "
                                "grid), fit 5" if detector else
                                "Poisson rows: 32-512 patterns of 512^2 or 1024^2 (50/50), 8 layouts "
                                "per size, 25-225 ROIs radius 24-48, fit 3-9"),
                   "rate_rows_per_s": rate, "duration_s": duration,
                   "hbm_arena_bytes_per_size": 24 << 30, "step_patterns": step_patterns,
                   "rows": "pinned rows read in place by the kernels" if in_place else
                           "row bands copied into the device arena by SM loads beside the steps"},
        "parity": {"max_abs_err_px": max(errs),
                   "rms_err_px": float(np.sqrt(np.concatenate(sq).mean())),
                   "vs": "FP64 oracle, one row per size"},
        "clocks": clk.summary()}


def run_cli_config(args):
    """The reference's command line end to end (src/main.cpp, src/process_files.hpp):
    1024^2 16-bit TIFFs on tmpfs (16 distinct patterns listed in turn), 100 ROIs
    of 64^2, FFT, float, fit 5, batch 32, 8 loader threads, text to /dev/null.
    Each run is a whole process; the pattern rate comes from a long and a short
    run, whose difference cancels the fixed start-up (CUDA context, reference
    spectra)."""
    import shutil
    import tempfile
    import __graft_entry__
    __graft_entry__.build_library()  # the library and the command line
    from emida_gb300 import synth
    cli = os.path.join(ROOT, "emida_gb300", "bin", "emida")
    tmp = tempfile.mkdtemp(dir="/dev/shm" if os.path.isdir("/dev/shm") else None)
    try:
        synth.write_tiff(os.path.join(tmp, "ref.tif"), synth.reference_pattern(1024, 7))
        uniq, _ = synth.deformed_patterns(1024, 7, 16, sigma_eps=5e-3)
        names = [os.path.join(tmp, f"def_{i}.tif") for i in range(16)]
        for n, p in zip(names, uniq):
            synth.write_tiff(n, p)
        mids, _ = synth.roi_grid(1024, 10, 32, margin=40)
        synth.write_roi_file(os.path.join(tmp, "roi.txt"), 32, mids)
        long_n, short_n = 8192, 512
        for n in (long_n, short_n):
            synth.write_deformed_list(os.path.join(tmp, f"def_{n}.txt"),
                                      [(float(i), 0.0, names[i % 16]) for i in range(n)])

        def run(n, extra):
            cmd = [cli, "-i", os.path.join(tmp, "ref.tif"), "-d", os.path.join(tmp, f"def_{n}.txt"),
                   "-b", os.path.join(tmp, "roi.txt"), "--precision", "float", "-f", "5",
                   "--crosspolicy", "fft", "--batchsize", "32", "--loadworkers", "8"] + extra
            t0 = time.perf_counter()
            r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
            if r.returncode != 0:
                raise RuntimeError(r.stderr[-500:])
            return time.perf_counter() - t0

        out = {}
        for key, extra in (("offsets", []), ("offsets_and_coefs", ["-q"])):
            run(short_n, extra)  # page cache and driver warm
            ts = statistics.median(run(short_n, extra) for _ in range(3))
            tl = statistics.median(run(long_n, extra) for _ in range(3))
            rate = (long_n - short_n) / (tl - ts)
            out[key] = {"patterns_per_s": rate, "pairs_per_s": rate * len(mids),
                        f"wall_s_{long_n}": tl, f"wall_s_{short_n}": ts,
                        "startup_s": max(0.0, ts - short_n / rate)}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    print(json.dumps({
        "metric": "patterns/s through the emida command line, TIFF files in, text out",
        "value": out["offsets"]["patterns_per_s"], "unit": "patterns/s", "n_gpus": 1,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "1024^2 uint16 TIFFs (16 distinct, listed in turn) on tmpfs, 100 ROIs "
                               "of 64^2, --crosspolicy fft --precision float -f 5 --batchsize 32 "
                               "--loadworkers 8, text to /dev/null",
                   "patterns": [short_n, long_n]},
        "runs": out}), flush=True)


def run_precision(args):
    """2048 patterns of 1024^2, 100 ROIs r=32 (10 x 10 grid), fit size 7: the
    brute policy's 127 x 127-lag correlation as a BF16 hi/lo contraction on the
    tcgen05 tensor cores (FP64 sums, means and fit) beside the FP32 fused FFT,
    both against the FP64 brute oracle (the reference's --precision double)."""
    import ctypes
    import __graft_entry__
    __graft_entry__.build_library()
    from emida_gb300 import DeviceBuffer, GpuOffset, _lib
    from oracle import oracle as eo
    P, s = 2048, 7
    ref, uniq, begins = workload()
    S = len(begins)
    pairs = P * S
    pat = 1024 * 1024 * 2
    d_pics = DeviceBuffer(P * pat)
    d_uniq = DeviceBuffer.from_array(uniq)
    for k in range(P // UNIQUE):  # the 32 distinct patterns repeated, on the device
        _lib.call("emida_gb_memcpy_d2d", ctypes.c_void_p(d_pics.ptr.value + k * UNIQUE * pat),
                  d_uniq.ptr, UNIQUE * pat)
    if args.profile_case:  # a few launches of the tensor form only (for ncu)
        g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "brute", s, 1, "float",
                      np.uint16, "tensor")
        g.allocate_memory(ref)
        d_offs = DeviceBuffer(args.profile_case * S * 16)
        for _ in range(3):
            g.run_device(d_pics, args.profile_case, d_offs)
        _lib.call("emida_gb_synchronize")
        print(json.dumps({"profile_case_patterns": args.profile_case, "mode": g.mode}))
        g.close()
        return
    # the staged FP32 brute form (CUDA cores, the reference's kernels) on a slice
    n_plain = 32
    gp = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "brute", s, 1, "float",
                   np.uint16, "plain")
    gp.allocate_memory(ref)
    d_po = DeviceBuffer(n_plain * S * 16)
    gp.run_device(d_pics, n_plain, d_po)
    plain_ms = gp.time_device(d_pics, n_plain, d_po, 2) / 2
    plain = {"value": n_plain * S / (plain_ms / 1000.0), "ms_per_step": plain_ms * P / n_plain,
             "sample": f"{n_plain} patterns, scaled to {P}"}
    gp.close()
    n_check = 2
    o_offs, o_coefs, o_peaks = eo.get_offsets(ref, uniq[:n_check], begins, 64, 64, eo.POLICY_BRUTE, s)
    ok = well_posed(o_coefs, s)
    peak, peak_kind = (json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("bf16_tflops"),
                       "measured") if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) \
        else (1900.0, "fallback")
    forms = {}
    for name, policy, mode in (("tensor", "brute", "tensor"), ("fft", "fft", "fused")):
        g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, policy, s, 1, "float",
                      np.uint16, mode)
        g.allocate_memory(ref)
        d_offs, d_coefs = DeviceBuffer(pairs * 16), DeviceBuffer(pairs * 48)
        d_maxes = DeviceBuffer(pairs * 8)
        g.run_device(d_pics, P, d_offs, d_coefs, d_maxes)
        _lib.call("emida_gb_synchronize")
        offs = d_offs.download(np.float64, (pairs, 2))[:n_check * S]
        idx = d_maxes.download(np.dtype([("data", "<f4"), ("index", "<u4")]), pairs)["index"][:n_check * S]
        if mode == "fused":  # FFT map index -> lag-window index of the brute map
            qx, qy = idx % 128, idx // 128
            idx = ((qx + 63) % 128) + 127 * ((qy + 63) % 128)
        d = np.abs(offs - o_offs)
        for _ in range(args.warmup):
            g.run_device(d_pics, P, d_offs)
        _lib.call("emida_gb_synchronize")
        with ClockSampler(0) as clk:
            ms = g.time_device(d_pics, P, d_offs, args.steps) / args.steps
        forms[name] = {
            "value": pairs / (ms / 1000.0), "ms_per_step": ms, "form": g.mode,
            "peak_match_rate": float(np.mean(idx == o_peaks)),
            "max_abs_err_px": float(d[ok].max()), "rms_err_px": float(np.sqrt(np.mean(d[ok] ** 2))),
            "clocks": clk.summary(), "launches_per_step": g.launches_per_run(),
        }
        g.close()
    t = forms["tensor"]
    useful = 2.0 * 64 ** 4            # sum over lags of the overlap products
    issued = 3 * 2.0 * 128 * 128 * 4096  # three split products of the 128 x 128 x 4096 GEMM
    sec = t["ms_per_step"] / 1000.0
    line = {
        "metric": "ROI pairs/s, brute 127x127 lags as a BF16 hi/lo tensor-core contraction",
        "value": t["value"], "unit": "ROI pairs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3->f32", "data": "synthetic",
        "config": {"workload": "2048 x 1024^2 uint16 patterns, 100 ROIs r=32 (64x64), brute "
                               "127x127 lags, s=7", "patterns": P, "rois": S, "fitsize": s,
                   "l2": "inputs larger than L2 (4 GiB of patterns)"},
        "parity": {"vs": f"FP64 brute oracle, first {n_check} patterns ({n_check * S} pairs)",
                   "well_posed_fits": int(ok[:, 0].sum()), "tensor": {k: t[k] for k in (
                       "peak_match_rate", "max_abs_err_px", "rms_err_px")},
                   "fft_fp32": {k: forms["fft"][k] for k in ("peak_match_rate", "max_abs_err_px",
                                                             "rms_err_px")}},
        "roofline": {"bound": "tensor", "achieved": pairs * issued / sec / 1e12, "peak": peak,
                     "unit": "TFLOP/s", "frac": pairs * issued / sec / 1e12 / peak,
                     "peak_kind": peak_kind, "traffic": None,
                     "note": "issued BF16 MMA flops (3 x 2 x 128 x 128 x 4096 per pair) vs the "
                             "bf16 GEMM peak; useful flops are 2 x 64^4 per pair"},
        "useful_tflops": pairs * useful / sec / 1e12,
        "fft_fp32": {k: forms["fft"][k] for k in ("value", "ms_per_step", "form")},
        "plain_brute_fp32": plain,
        "gpu_launches": t["launches_per_step"] * args.steps,
        "clocks": t["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_profile_target(args):
    """Small cases of the 256-point cluster kernel, of the deformation fit and
    of the ingest modes for ncu: a few launches, then one timing line."""
    import ctypes
    import __graft_entry__
    __graft_entry__.build_library()
    from emida_gb300 import DeviceBuffer, GpuOffset, _lib, pinned_array, synth
    n = args.profile_case
    if args.profile_target == "inplace":
        ref, uniq, begins = workload()
        host = pinned_array((n, 1024, 1024))
        host[:] = np.resize(uniq, (n, 1024, 1024))
        g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "fft", 5, 1, "float",
                      np.uint16, "fused")
        g.allocate_memory(ref)
        o = DeviceBuffer(n * len(begins) * 16)
        for _ in range(3):
            g.run_device(host.ctypes.data, n, o)
        _lib.call("emida_gb_synchronize")
        t0 = time.perf_counter()
        for _ in range(3):
            g.run_device(host.ctypes.data, n, o)
        _lib.call("emida_gb_synchronize")
        ms = (time.perf_counter() - t0) * 1000 / 3
        print(json.dumps({"profile_target": "inplace", "patterns": n, "ms": ms,
                          "pairs_per_s": n * len(begins) / (ms / 1000)}))
        g.close()
        return
    if args.profile_target == "ingest":
        ref, uniq, begins = workload()
        host = pinned_array((n, 1024, 1024))
        host[:] = np.resize(uniq, (n, 1024, 1024))
        g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "fft", 5, 3, "float",
                      np.uint16, "fused")
        g.allocate_memory(ref)
        out = {"profile_target": "ingest", "patterns": n}
        for mode in ("copy", "gather", "sm_copy"):
            g.ingest = mode
            t0 = time.perf_counter()
            pending = []
            for b in range(0, n, 32):
                if len(pending) == 3:
                    g.wait(pending.pop(0))
                pending.append(g.submit(host[b:b + 32]))
            for t in pending:
                g.wait(t)
            out[mode + "_ms"] = (time.perf_counter() - t0) * 1000
        print(json.dumps(out))
        g.close()
        return
    if args.profile_target in ("fused64", "fused96", "fused192"):
        side = {"fused64": 32, "fused96": 48, "fused192": 96}[args.profile_target]
        ref = synth.reference_pattern(1024, 5)
        uniq, _ = synth.deformed_patterns(1024, 5, 8, sigma_eps=5e-3)
        _, begins = synth.roi_grid(1024, 10, side // 2, margin=side // 2 + 8)
        pics = np.ascontiguousarray(np.resize(uniq, (n, 1024, 1024)))
        g = GpuOffset((1024, 1024), begins, (side, side), (2 * side - 1, 2 * side - 1), 32, "fft", 5,
                      1, "float", np.uint16, "fused")
        g.allocate_memory(ref)
        d, o = DeviceBuffer.from_array(pics), DeviceBuffer(n * len(begins) * 16)
        for _ in range(3):
            g.run_device(d, n, o)
        _lib.call("emida_gb_synchronize")
        ms = g.time_device(d, n, o, 5) / 5
        print(json.dumps({"profile_target": args.profile_target, "pairs": n * len(begins), "ms": ms,
                          "pairs_per_s": n * len(begins) / (ms / 1000)}))
        g.close()
        return
    if args.profile_target == "cluster":
        ref = synth.reference_pattern(1024, 5)
        uniq, _ = synth.deformed_patterns(1024, 5, 8, sigma_eps=5e-3)
        _, begins = synth.roi_grid(1024, 6, 64, margin=80)
        pics = np.ascontiguousarray(np.resize(uniq, (n, 1024, 1024)))
        g = GpuOffset((1024, 1024), begins, (128, 128), (255, 255), 8, "fft", 5, 1, "float",
                      np.uint16, "fused")
        g.allocate_memory(ref)
        d, o = DeviceBuffer.from_array(pics), DeviceBuffer(n * len(begins) * 16)
        for _ in range(3):
            g.run_device(d, n, o)
        _lib.call("emida_gb_synchronize")
        ms = g.time_device(d, n, o, 5) / 5
        print(json.dumps({"profile_target": "cluster", "pairs": n * len(begins), "ms": ms}))
        g.close()
        return
    rng = np.random.default_rng(1)
    axis = np.linspace(60, 964, 10)
    mids = np.array([(x, y) for y in axis for x in axis])
    offs = rng.normal(0, 1.0, (n, len(mids), 2))
    dm, do, dout = DeviceBuffer.from_array(mids), DeviceBuffer.from_array(offs), DeviceBuffer(n * 72)
    c = (ctypes.c_double * 3)(512.0, 512.0, 512.0)
    args_c = (dm.ptr, do.ptr, len(mids), n, c, None, 0.0, dout.ptr)
    for _ in range(2):
        _lib.call("emida_gb_fit_homography", *args_c, None)
    _lib.call("emida_gb_synchronize")
    ms = ctypes.c_float()
    _lib.call("emida_gb_time_fit_homography", *args_c, 5, ctypes.byref(ms))
    print(json.dumps({"profile_target": "homography", "patterns": n, "ms": ms.value / 5}))


def parity_vs_oracle(offs, peaks, ref, pics, begins, policy, s, cross=None):
    """Max and RMS |offset - FP64 oracle| over well-posed fits, and the peak
    match rate, for the results of `pics`."""
    from oracle import oracle as eo
    pol = eo.POLICY_FFT if policy == "fft" else eo.POLICY_BRUTE
    cw = cross or 127
    o_offs, o_coefs, o_peaks = eo.get_offsets(ref, pics, begins, 64, 64, pol, s, cw, cw)
    ok = well_posed(o_coefs, s)
    d = np.abs(offs[:len(o_offs)] - o_offs)[ok]
    return {"max_abs_err_px": float(d.max()), "rms_err_px": float(np.sqrt(np.mean(d ** 2))),
            "peak_match_rate": float(np.mean(peaks[:len(o_peaks)] == o_peaks)),
            "checked_pairs": len(o_offs)}


def reference_plain(ref, pics, begins, precision, repeats):
    """The reference's own staged GPU pipeline (its gpu_offset<T, uint16_t> with
    cuFFT, src/gpu_offset.hpp:234-316) on the same job: device-resident
    (get_offset_core over batches already in its input buffers) and end to
    end (transfer, get_offset_core and finalize per batch from pinned memory)."""
    from oracle import ref_gpu
    if not ref_gpu.available():
        return {"unavailable": "the reference's sources are not staged into baseline/_ref"}
    P, S = len(pics), len(begins)
    nb = P // 32
    batches = []
    for b in range(nb):
        h = pinned_u16((32, 1024, 1024))
        h[:] = pics[b * 32:(b + 1) * 32]
        batches.append(h)
    g = ref_gpu.RefGpuOffset(ref, begins, 64, 32, "fft", 5, precision, in_buffers=nb)
    offs, _, peaks = g.run_batch(batches[0])
    par = parity_vs_oracle(offs, peaks, ref, pics[:2], begins, "fft", 5)
    g.time_core(batches, 1)
    ms = g.time_core(batches, repeats) / repeats
    e2e_ms = min(g.time_e2e(batches) for _ in range(2))
    g.close()
    return {"value": P * S / (ms / 1000.0), "ms_per_step": ms,
            "e2e": {"value": P * S / (e2e_ms / 1000.0), "ms_per_step": e2e_ms},
            "parity": par, "precision": precision,
            "what": "the reference's gpu_offset<T, uint16_t> compiled unmodified with its six kernel "
                    "files and cuFFT for sm_103a: value = get_offset_core per 32-pattern batch on "
                    "batches already in device memory (host wall time, as it synchronises the "
                    "device twice per batch); e2e = transfer_pic_to_device_async, get_offset_core "
                    "and finalize per batch from pinned memory"}


def fp64_leg(ref, pics, begins, d_pics, steps, warmup):
    """The detector job in float64 on the fused form, beside the reference's
    own staged pipeline in float64."""
    from emida_gb300 import DeviceBuffer, GpuOffset, _lib
    P, S = len(pics), len(begins)
    g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "fft", 5, 1, "double", np.uint16, "fused")
    g.allocate_memory(ref)
    d_o, d_c, d_m = DeviceBuffer(P * S * 16), DeviceBuffer(P * S * 48), DeviceBuffer(P * S * 16)
    g.run_device(d_pics, P, d_o, d_c, d_m)
    _lib.call("emida_gb_synchronize")
    offs = d_o.download(np.float64, (P * S, 2))
    peaks = d_m.download(g.data_index, P * S)["index"]
    par = parity_vs_oracle(offs, peaks, ref, pics[:2], begins, "fft", 5)
    for _ in range(warmup):
        g.run_device(d_pics, P, d_o)
    _lib.call("emida_gb_synchronize")
    with ClockSampler(0) as clk:
        ms = g.time_device(d_pics, P, d_o, steps) / steps
    g.close()
    flop = P * S * (5 * 128 * 128 * 14 + 6 * 65 * 128 + 3 * 64 * 64)
    plain = reference_plain(ref, pics, begins, "double", 2)
    out = {"value": P * S / (ms / 1000.0), "ms_per_step": ms, "form": "fused", "parity": par,
           "compute": {"fp64_tflops": flop / (ms / 1000.0) / 1e12, "fp64_peak_tflops_nominal": 1.25,
                       "frac": flop / (ms / 1000.0) / 1e12 / 1.25},
           "plain_reference": plain, "clocks": clk.summary()}
    if "value" in plain:
        out["over_plain_reference"] = out["value"] / plain["value"]
    return out


def tensor_leg(ref, pics, begins, d_pics, steps, warmup, s=7):
    """The brute policy's 127 x 127-lag correlation on the tcgen05 tensor cores
    (BF16 hi/lo split, FP32 accumulation; FP64 sums and fit) over the same job
    at fit size 7, with the useful-flop roofline against a third of the
    measured BF16 peak (the split issues three products)."""
    from emida_gb300 import DeviceBuffer, GpuOffset, _lib
    P, S = len(pics), len(begins)
    g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "brute", s, 1, "float", np.uint16,
                  "tensor")
    g.allocate_memory(ref)
    d_o, d_m = DeviceBuffer(P * S * 16), DeviceBuffer(P * S * 8)
    g.run_device(d_pics, P, d_o, None, d_m)
    _lib.call("emida_gb_synchronize")
    offs = d_o.download(np.float64, (P * S, 2))
    peaks = d_m.download(g.data_index, P * S)["index"]
    par = parity_vs_oracle(offs, peaks, ref, pics[:2], begins, "brute", s)
    for _ in range(warmup):
        g.run_device(d_pics, P, d_o)
    _lib.call("emida_gb_synchronize")
    with ClockSampler(0) as clk:
        ms = g.time_device(d_pics, P, d_o, steps) / steps
    launches = g.launches_per_run()
    g.close()
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    bf16, kind = (json.load(open(mp)).get("bf16_tflops"), "measured") if os.path.exists(mp) else (1900.0, "fallback")
    useful = P * S * 2.0 * 64 ** 4 / (ms / 1000.0) / 1e12
    issued = P * S * 3 * 2.0 * 128 * 128 * 4096 / (ms / 1000.0) / 1e12
    return {"value": P * S / (ms / 1000.0), "ms_per_step": ms, "fitsize": s, "parity": par,
            "roofline": {"bound": "tensor", "achieved": useful, "peak": bf16 / 3, "unit": "TFLOP/s",
                         "frac": useful / (bf16 / 3), "peak_kind": kind,
                         "note": "useful flops (2 x 64^4 per pair) against a third of the bf16 burst "
                                 "peak, as the hi/lo split issues three products"},
            "issued_tflops": issued, "launches_per_step": launches, "clocks": clk.summary()}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.config == "batching":
        return run_batching(args)
    if args.config == "serving":
        return run_serving(args)
    if args.config == "precision":
        return run_precision(args)
    if args.config == "cli":
        return run_cli_config(args)
    if args.profile_case and args.profile_target != "fused":
        return run_profile_target(args)

    import __graft_entry__
    __graft_entry__.build_library()
    from emida_gb300 import DeviceBuffer, GpuOffset, _lib

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import ctypes
    _lib.call("emida_gb_set_device", local)  # the library keeps its own current device

    ref, uniq, begins = workload()
    P = args.patterns
    S = len(begins)
    pics = np.ascontiguousarray(np.resize(uniq, (P, 1024, 1024)))
    pairs_per_step = P * S
    g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "fft", 5, args.in_flight, args.precision,
                  np.uint16, args.mode)
    g.allocate_memory(ref)
    d_pics = DeviceBuffer.from_array(pics)
    d_offs = DeviceBuffer(pairs_per_step * 2 * 8)
    d_coefs = DeviceBuffer(pairs_per_step * 6 * 8)

    if args.profile_case:
        n = args.profile_case
        for _ in range(3):
            g.run_device(d_pics, n, d_offs)
        _lib.call("emida_gb_synchronize")
        print(json.dumps({"profile_case_patterns": n, "mode": g.mode}))
        return

    # parity gate on the bench data: the first pattern against the FP64 oracle
    from oracle import oracle as eo
    d_maxes = DeviceBuffer(pairs_per_step * 16)
    g.run_device(d_pics, P, d_offs, d_coefs, d_maxes)
    _lib.call("emida_gb_synchronize")
    offs = d_offs.download(np.float64, (pairs_per_step, 2))
    peaks = d_maxes.download(g.data_index, pairs_per_step)["index"][:2 * S]
    o_offs, o_coefs, o_peaks = eo.get_offsets(ref, pics[:2], begins, 64, 64, eo.POLICY_FFT, 5)
    peak_match = float(np.mean(peaks == o_peaks))
    ok = well_posed(o_coefs, 5)
    d = np.abs(offs[:2 * S] - o_offs)
    err = float(d[ok].max())
    tol = 1e-2
    assert err <= tol, f"offset error {err} px exceeds {tol}"
    rms = float(np.sqrt(np.mean(d[ok] ** 2)))

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        g.run_device(d_pics, P, d_offs, d_coefs)
    _lib.call("emida_gb_synchronize")
    barrier()
    with ClockSampler(local) as clk:
        ms = g.time_device(d_pics, P, d_offs, args.steps)
    _lib.call("emida_gb_synchronize")
    barrier()
    ms = max_over_ranks(ms, dist, device="cuda")
    ms_step = ms / args.steps
    value = whole_job_rate(pairs_per_step, ms_step / 1000.0, world)

    # per-launch duration of the dominant kernel (fused: one launch per step)
    launches = g.launches_per_run()
    roof_bytes = pairs_per_step * (64 * 64 * 2 + 16) + S * 65 * 128 * (8 if args.precision == "float" else 16)
    peak, peak_kind = measured_peaks()
    achieved = roof_bytes / (ms_step / 1000.0) / 1e9
    flop = pairs_per_step * (5 * 128 * 128 * 14 + 6 * 65 * 128 + 3 * 64 * 64)
    sm_max = 2070.0
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    # the arithmetic pipe of the chosen precision: FP32 lanes at the maximum SM
    # clock, or GB300's nominal FP64 rate (no measured FP64 peak is available)
    fpu, fpu_peak = ("fp32", fp32_peak) if args.precision == "float" else ("fp64", 1.25)

    # the deformation fit after the path (python/process_offsets.py:83-104) on
    # this job's offsets, with the fit-quality mask: one projective map per pattern
    mids = (np.asarray(begins, dtype=np.float64) + 32.0)
    d_mids = DeviceBuffer.from_array(np.ascontiguousarray(mids))
    d_f = DeviceBuffer(P * 9 * 8)
    centre = (ctypes.c_double * 3)(512.0, 512.0, 512.0)
    g.run_device(d_pics, P, d_offs, d_coefs)
    _lib.call("emida_gb_synchronize")
    fit_args = (d_mids.ptr, d_offs.ptr, S, P, centre, d_coefs.ptr, 1e-6, d_f.ptr)
    _lib.call("emida_gb_time_fit_homography", *fit_args, 2, ctypes.byref(ctypes.c_float()))
    fit_ms = ctypes.c_float()
    _lib.call("emida_gb_time_fit_homography", *fit_args, 10, ctypes.byref(fit_ms))
    deformation = {"patterns_per_s": P / (fit_ms.value / 10 / 1000.0), "ms_per_step": fit_ms.value / 10,
                   "what": "per pattern a 3x3 projective map from its 100 ROI offsets "
                           "(FP64 Householder QR of the 200 x 9 system and a one-sided Jacobi SVD of "
                           "its 9 x 9 triangle; a warp per pattern, or a half-warp per pattern in the SVD "
                           "from two patterns per SM on)"}

    # plain form on the same data for the fused-vs-plain ratio
    plain = None
    if args.mode == "fused" and not args.no_plain:
        gp = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 32, "fft", 5, 1, args.precision,
                       np.uint16, "plain")
        gp.allocate_memory(ref)
        gp.run_device(d_pics, P, d_offs)
        pm = gp.time_device(d_pics, P, d_offs, max(2, args.steps // 4)) / max(2, args.steps // 4)
        plain = {"value": pairs_per_step / (pm / 1000.0), "ms_per_step": pm,
                 "launches_per_step": gp.launches_per_run() * (P // 32)}
        gp.close()

    # end to end through the C ABI from pinned host memory: submit/wait keeps
    # up to three batches in flight, so the copy of batch b+1 overlaps the
    # path on batch b (input, compute and output streams)
    hbuf = ctypes.c_void_p()
    _lib.call("emida_gb_malloc_host", ctypes.byref(hbuf), pics.nbytes)
    ctypes.memmove(hbuf, pics.ctypes.data, pics.nbytes)
    host_offs = np.zeros((pairs_per_step, 2))
    e2e_steps = max(4, args.steps // 2)
    nb = P // 32
    in_flight = args.in_flight

    def e2e_run(steps):
        # `steps` passes over the job as one stream of batches, as a scan is
        # processed: up to in_flight batches in flight across step boundaries;
        # every batch's copy, path and results lie inside the run
        pending = []
        for i in range(steps * nb):
            if len(pending) == in_flight:
                t, k = pending.pop(0)
                host_offs[k * 32 * S:(k + 1) * 32 * S] = g.wait(t)[0]
            pending.append((g.submit(hbuf.value + (i % nb) * 32 * 1024 * 1024 * 2), i % nb))
        for t, k in pending:
            host_offs[k * 32 * S:(k + 1) * 32 * S] = g.wait(t)[0]

    def e2e_time(steps):
        barrier()
        t0 = time.perf_counter()
        e2e_run(steps)
        barrier()
        return max_over_ranks((time.perf_counter() - t0) * 1000 / steps, dist, device="cuda")

    # the library's default ingest for this form: the row bands copied by SM
    # loads on a few CTAs beside the path
    default_ingest = g.ingest
    e2e_run(1)
    assert np.array_equal(host_offs, offs), "e2e offsets differ from the device-resident run"
    e2e_ms = e2e_time(e2e_steps)
    e2e_value = whole_job_rate(pairs_per_step, e2e_ms / 1000.0, world)
    # one step alone, the pipeline filled and drained inside it
    e2e_one_ms = statistics.median(e2e_time(1) for _ in range(3))
    # the other ingest modes: kernels reading the ROI pixels in place (no
    # copy), a gather kernel packing the ROI rows
    # beside the path, and the row bands copied by SM loads
    ingest = {}
    for mode in ("copy", "in_place", "gather", "sm_copy"):
        if mode == default_ingest:
            continue
        g.ingest = mode
        if g.ingest != mode:
            continue
        e2e_run(1)
        assert np.array_equal(host_offs, offs), f"{mode} offsets differ from the device-resident run"
        m_ms = e2e_time(e2e_steps)
        one_ms = statistics.median(e2e_time(1) for _ in range(3))
        ingest[mode] = {"value": whole_job_rate(pairs_per_step, m_ms / 1000.0, world), "ms_per_step": m_ms,
                        "one_step_ms": one_ms}
    g.ingest = default_ingest
    _lib.call("emida_gb_free_host", hbuf)

    # the reference's own staged GPU pipeline on the same job (the plain
    # baseline of the fused/plain ratio), and the other legs of the path
    legs = {}
    if rank == 0 and world == 1 and not args.no_legs:
        legs["plain_reference"] = reference_plain(ref, pics, begins, args.precision, 3)
        if "value" in legs["plain_reference"]:
            legs["over_plain_reference"] = {
                "value": value / legs["plain_reference"]["value"],
                "e2e": e2e_value / legs["plain_reference"]["e2e"]["value"],
                "target": 5.0}
        if args.precision == "float" and args.mode == "fused":
            legs["fp64"] = fp64_leg(ref, pics, begins, d_pics, max(5, args.steps // 5), args.warmup)
            legs["tensor"] = tensor_leg(ref, pics, begins, d_pics, max(5, args.steps // 5), args.warmup)
            # 8 s of arrivals, as the serving config runs: the p99 of about 800 rows
            # is not set by a single pause of the host's loop thread
            legs["serving"] = serving_measure("float", "detector", 100.0, 8.0, 128, False)
            bm = batching_measure("float", 5, args.warmup)
            legs["batching"] = {k: bm[k] for k in ("metric", "value", "unit", "ms_per_step", "config",
                                                  "autotune", "parity", "clocks")}

    cpu = port = None
    if rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        cr = CpuReference(ref, uniq, begins, args.precision)
        v, pairs, dt = cr.run(10.0, threads)
        what = ("the reference's own CPU code (sums_serial, cross_corr_serial over 127x127 lags, "
                f"subpixel_max_serial) in {args.precision}" if cr.kind == "reference" else
                "the oracle's FP64 C restatement, FFT policy")
        cpu = {"value": v, "unit": "ROI pairs/s", "cores": threads, "kind": cr.kind,
               "sample": f"{pairs} ROI pairs in {dt:.1f} s on all host cores: {what}"}
        if cr.kind == "reference":
            v2, pairs2, dt2 = cpu_port(ref, uniq, begins, 5.0, threads)
            port = {"value": v2, "unit": "ROI pairs/s", "cores": threads, "kind": "port",
                    "sample": f"{pairs2} ROI pairs in {dt2:.1f} s: the oracle's FP64 C restatement "
                              "of the FFT policy (no CPU FFT path exists in the reference)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "ROI pairs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "float" else "f64", "data": "synthetic",
            "config": detector_config(P, S, world, args.precision),
            "form": g.mode,
            "parity": {"max_abs_err_px": err, "rms_err_px": rms, "tol_px": tol,
                       "peak_match_rate": peak_match,
                       "vs": "FP64 oracle, first two patterns", "well_posed_fits": int(ok.sum()),
                       "extrapolated_fits": int((~ok).sum())},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": (TRAFFIC_PER_PAIR * pairs_per_step + TRAFFIC_PER_LAUNCH
                                     if g.mode == "fused" and args.precision == "float" else None),
                         "note": "FP32 pipe / shared memory bound; see compute"},
            "compute": {f"{fpu}_tflops": flop / (ms_step / 1000.0) / 1e12,
                        f"{fpu}_peak_tflops_nominal": fpu_peak,
                        "frac": flop / (ms_step / 1000.0) / 1e12 / fpu_peak,
                        "flop_per_pair": flop // pairs_per_step},
            "plain": plain,
            **legs,
            "deformation_fit": deformation,
            "cpu_baseline": cpu,
            "cpu_port_fft": port,
            "e2e": {"value": e2e_value, "unit": "ROI pairs/s",
                    "h2d_bytes_per_step": int(P * roi_rows(begins, 64) * 1024 * 2),
                    "d2h_bytes_per_step": pairs_per_step * (16 + 48 + 8),
                    "ms_per_step": e2e_ms,
                    "steps": e2e_steps,
                    "one_step_ms": e2e_one_ms,
                    "ingest": default_ingest,
                    "input": f"pinned host batches; the {roi_rows(begins, 64)} of 1024 rows that hold "
                             "ROI pixels are copied, " + INGEST_HOW.get(default_ingest, default_ingest),
                    "pipeline": f"the steps run as one stream of {nb}-batch passes through submit/wait, "
                                f"{in_flight} batches of 32 in flight across step boundaries; "
                                "one_step_ms: a single step with the pipeline filled and drained in it"},
            "e2e_ingest": ingest,
            "gpu_launches": launches * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    g.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
