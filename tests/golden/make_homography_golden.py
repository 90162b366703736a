#!/usr/bin/env python3
"""Golden vectors for the deformation-gradient (projective) fit downstream of
the path, made by running the reference's own python/process_offsets.py.

Run where the reference is mounted (its path is the first argument, or the
EMIDA_REFERENCE environment variable).  The script is fed seeded synthetic ROI
offsets in the format it reads (a ROI count, then per pattern a name line and "x y dx dy" lines).  It
imports `pylab` only for numpy's names; a stand-in module that re-exports numpy
(printing at full precision) is put on its path, so the reference's own
arithmetic produces the recorded matrices.  Output: homography_golden.npz with
the inputs (mids, offsets, centre) and the printed UU / UU[2,2] per pattern.
"""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EMIDA_REFERENCE", "")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("usage: %s REFERENCE_TREE (or set EMIDA_REFERENCE)" % sys.argv[0])
N = 873  # process_offsets.py fixes the pattern size, hence the centre (436, 436, 436)

PYLAB = '''import sys
import numpy as np
from numpy import *
np.set_printoptions(precision=17, floatmode="unique", linewidth=400)
'''


def synth(seed=7, patterns=6, grid=10):
    """ROI centres on a grid; offsets from a near-identity projective map plus noise."""
    rng = np.random.default_rng(seed)
    c = N // 2
    axis = np.linspace(60, N - 60, grid).round()
    mids = np.array([(x, y) for y in axis for x in axis], dtype=np.float64)
    offsets = []
    for _ in range(patterns):
        Hm = np.eye(3)
        Hm[:2, :2] += rng.normal(0, 3e-3, (2, 2))
        Hm[:2, 2] = rng.normal(0, 2.0, 2)
        Hm[2, :2] = rng.normal(0, 2e-6, 2)
        p = np.stack([mids[:, 0] - c, mids[:, 1] - c, np.full(len(mids), c)], axis=1)
        q = p @ Hm.T
        new = q[:, :2] / q[:, 2:3] * c + c
        offsets.append(new - mids + rng.normal(0, 0.01, mids.shape))
    return mids, np.array(offsets)


def run_reference(mids, offsets):
    lines = [str(len(mids))]
    for k, off in enumerate(offsets):
        lines.append(f"pattern_{k}")
        lines += [" ".join(repr(float(v)) for v in (x, y, dx, dy)) for (x, y), (dx, dy) in zip(mids, off)]
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, "pylab.py"), "w") as f:
            f.write(PYLAB)
        env = dict(os.environ, PYTHONPATH=tmp)
        r = subprocess.run([sys.executable, os.path.join(REF, "python", "process_offsets.py")],
                           input="\n".join(lines) + "\n", capture_output=True, text=True, env=env,
                           check=True)
    mats = []
    for block in r.stdout.split("pattern_")[1:]:
        nums = re.findall(r"[-+]?\d+\.\d*(?:e[-+]?\d+)?|[-+]?\d+e[-+]?\d+", block.split("\n", 1)[1])
        mats.append(np.array([float(v) for v in nums[:9]]).reshape(3, 3))
    return np.array(mats)


def main():
    mids, offsets = synth()
    uu = run_reference(mids, offsets)
    assert uu.shape == (len(offsets), 3, 3), uu.shape
    np.savez(os.path.join(HERE, "homography_golden.npz"), mids=mids, offsets=offsets,
             centre=np.array([N // 2] * 3, dtype=np.float64), uu=uu)
    print("wrote homography_golden.npz:", uu.shape)


if __name__ == "__main__":
    main()
