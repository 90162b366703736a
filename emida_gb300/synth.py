"""Seeded synthetic EBSD-like patterns standing in for the reference's detector
data (FeAl patterns, not available here).

Reference pattern (from `seed`): a radial Gaussian background (sigma = 0.6 W,
peak 3000 counts) plus 12 Kikuchi-like bands, each a line at angle
theta ~ U[0, pi) and offset rho ~ U(-W/3, W/3) from the centre, with a Gaussian
cross-profile of width ~ U[8, 20] px and amplitude ~ U[400, 1200]; then
Poisson noise, clipped to uint16.  Deformed pattern i redraws the bands
through x' = (I + eps) x + t about the centre (eps_ij ~ N(0, sigma_eps),
t ~ U(-3, 3)^2 px) with fresh Poisson noise; its seed is seed * 1000 + i + 1.
ROI grids are n x n regular grids of centres from `margin` to W - margin,
written as top-left corners (mid - radius).
"""
import numpy as np


def _bands(seed, n=12):
    rng = np.random.default_rng(seed)
    theta = rng.uniform(0, np.pi, n)
    rho = rng.uniform(-1 / 3, 1 / 3, n)
    width = rng.uniform(8, 20, n)
    amp = rng.uniform(400, 1200, n)
    return theta, rho, width, amp


def _render(h, w, bands, A=None, t=(0.0, 0.0), noise_seed=None):
    theta, rho, width, amp = bands
    cy, cx = (h - 1) / 2.0, (w - 1) / 2.0
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    X, Y = xx - cx - t[0], yy - cy - t[1]
    if A is not None:
        inv = np.linalg.inv(A)
        X, Y = inv[0, 0] * X + inv[0, 1] * Y, inv[1, 0] * X + inv[1, 1] * Y
    r2 = (xx - cx) ** 2 + (yy - cy) ** 2
    img = 3000.0 * np.exp(-r2 / (2 * (0.6 * w) ** 2))
    for th, r, wd, a in zip(theta, rho, width, amp):
        d = X * np.cos(th) + Y * np.sin(th) - r * w
        img += a * np.exp(-(d * d) / (2 * wd * wd))
    rng = np.random.default_rng(noise_seed)
    return np.clip(rng.poisson(img), 0, 65535).astype(np.uint16)


def reference_pattern(size, seed):
    w, h = (size, size) if np.isscalar(size) else size
    return _render(h, w, _bands(seed), noise_seed=seed)


def deformed_patterns(size, seed, count, sigma_eps=5e-3, first=0):
    """`count` deformed patterns [count][h][w] uint16 and their (A, t)."""
    w, h = (size, size) if np.isscalar(size) else size
    bands = _bands(seed)
    out = np.empty((count, h, w), dtype=np.uint16)
    truth = []
    for k in range(count):
        i = first + k
        rng = np.random.default_rng(seed * 1000 + i + 1)
        A = np.eye(2) + rng.normal(0, sigma_eps, (2, 2))
        t = rng.uniform(-3, 3, 2)
        out[k] = _render(h, w, bands, A, t, noise_seed=seed * 1000 + i + 1)
        truth.append((A, t))
    return out, truth


def roi_grid(size, n, radius, margin=40):
    """ROI top-left corners of an n x n grid of mids from margin to W - margin
    (mids clamped so every ROI stays inside the pattern)."""
    w, h = (size, size) if np.isscalar(size) else size
    xs = np.linspace(max(margin, radius), w - max(margin, radius), n).round().astype(int)
    ys = np.linspace(max(margin, radius), h - max(margin, radius), n).round().astype(int)
    mids = np.array([(x, y) for y in ys for x in xs], dtype=np.int64)
    return mids, (mids - radius).astype(np.uint32)


def random_layout(size, seed, radius, count, margin=8, tries=200000):
    """Non-overlapping ROI mids by rejection sampling (batching / serving layouts)."""
    w, h = (size, size) if np.isscalar(size) else size
    rng = np.random.default_rng(seed)
    mids = []
    for _ in range(tries):
        if len(mids) >= count:
            break
        x = int(rng.integers(radius + margin, w - radius - margin + 1))
        y = int(rng.integers(radius + margin, h - radius - margin + 1))
        if all(abs(x - a) >= 2 * radius or abs(y - b) >= 2 * radius for a, b in mids):
            mids.append((x, y))
    mids = np.array(mids, dtype=np.int64).reshape(-1, 2)
    return mids, (mids - radius).astype(np.uint32)


def write_roi_file(path, radius, mids):
    """The reference's --slicepos format: first line radius, then 'x y' mids
    (src/args_parser.cpp:67-111)."""
    with open(path, "w") as f:
        f.write(f"{radius}\n")
        for x, y in mids:
            f.write(f"{int(x)} {int(y)}\n")


def write_tiff(path, img, rows_per_strip=16):
    """A little-endian, uncompressed, single-channel 16-bit TIFF in strips: the
    kind the reference loads (src/load_tiff.hpp:14-53)."""
    import struct
    img = np.ascontiguousarray(img, dtype="<u2")
    h, w = img.shape
    data = img.tobytes()
    strips = [data[r * w * 2:min(h, r + rows_per_strip) * w * 2] for r in range(0, h, rows_per_strip)]
    n, entries = len(strips), 10
    offs_at = 8 + 2 + 12 * entries + 4
    counts_at = offs_at + 4 * n
    pos, offsets = counts_at + 4 * n, []
    for s in strips:
        offsets.append(pos)
        pos += len(s)

    def ent(tag, typ, count, value):
        if typ == 3 and count == 1:
            return struct.pack("<HHIHH", tag, typ, count, value, 0)
        return struct.pack("<HHII", tag, typ, count, value)

    out = b"II" + struct.pack("<HI", 42, 8) + struct.pack("<H", entries)
    out += ent(256, 4, 1, w) + ent(257, 4, 1, h) + ent(258, 3, 1, 16) + ent(259, 3, 1, 1)
    out += ent(262, 3, 1, 1) + ent(273, 4, n, offs_at) + ent(274, 3, 1, 1) + ent(277, 3, 1, 1)
    out += ent(278, 4, 1, rows_per_strip) + ent(279, 4, n, counts_at) + struct.pack("<I", 0)
    out += struct.pack(f"<{n}I", *offsets) + struct.pack(f"<{n}I", *[len(s) for s in strips])
    with open(path, "wb") as f:
        f.write(out + b"".join(strips))


def write_deformed_list(path, entries):
    """The reference's --deformed list: 'x y path' lines (src/process_files.hpp:56-75)."""
    with open(path, "w") as f:
        for x, y, name in entries:
            f.write(f"{x} {y} {name}\n")
