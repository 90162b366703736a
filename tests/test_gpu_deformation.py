"""The deformation fit after the path (python/process_offsets.py:83-104) on the
GPU: FP64 QR and one-sided Jacobi SVD per pattern against the reference script's own
output, against the oracle (scipy's SVD, as the reference calls it), with the
quality mask of jove/analyze.py, and on offsets computed by the path."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def synth(seed, patterns, grid=10, n=873, noise=0.01):
    rng = np.random.default_rng(seed)
    c = n // 2
    axis = np.linspace(60, n - 60, grid).round()
    mids = np.array([(x, y) for y in axis for x in axis], dtype=np.float64)
    offs = []
    for _ in range(patterns):
        h = np.eye(3)
        h[:2, :2] += rng.normal(0, 3e-3, (2, 2))
        h[:2, 2] = rng.normal(0, 2.0, 2)
        h[2, :2] = rng.normal(0, 2e-6, 2)
        p = np.stack([mids[:, 0] - c, mids[:, 1] - c, np.full(len(mids), c)], axis=1) @ h.T
        offs.append(p[:, :2] / p[:, 2:3] * c + c - mids + rng.normal(0, noise, mids.shape))
    return mids, np.array(offs), np.array([c, c, c], dtype=np.float64)


def test_matches_reference_script_output():
    from emida_gb300 import fit_homography
    g = np.load(os.path.join(GOLDEN, "homography_golden.npz"))
    got = fit_homography(g["mids"], g["offsets"], g["centre"])
    assert np.allclose(got, g["uu"], rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("grid,patterns", [(3, 40), (10, 701), (20, 40), (20, 400), (30, 7), (40, 5)])
def test_matches_oracle(grid, patterns):
    # two patterns share a warp from two patterns per SM on, up to about 780
    # ROIs (an odd count leaves the last warp's second half on a copy); fewer
    # patterns, and 900 or 1600 ROIs, run one per warp
    from emida_gb300 import fit_homography
    from oracle import oracle as eo
    mids, offs, centre = synth(11 + grid, patterns, grid=grid)
    got = fit_homography(mids, offs, centre)
    for k in range(len(offs)):
        assert np.allclose(got[k], eo.homography_fit(mids, offs[k], centre), rtol=1e-9, atol=1e-13)


def test_quality_mask():
    from emida_gb300 import fit_homography
    from oracle import oracle as eo
    mids, offs, centre = synth(5, 6)
    rng = np.random.default_rng(9)
    coefs = rng.normal(0, 1, (len(offs), len(mids), 6))
    coefs[..., 3] = -1.0
    coefs[..., 5] = -1.0
    coefs[..., 4] = 0.1
    bad = rng.random((len(offs), len(mids))) < 0.3
    coefs[bad, 3] = 1.0  # det of the negated quadratic < 0: not a maximum
    coefs[-1, :95, 3] = 1.0  # the last pattern keeps only five ROIs
    got = fit_homography(mids, offs, centre, coefs=coefs, min_det=1e-6)
    for k in range(len(offs) - 1):
        keep = ~bad[k]
        assert np.allclose(got[k], eo.homography_fit(mids[keep], offs[k][keep], centre), rtol=1e-9,
                           atol=1e-13)
    assert np.isnan(got[-1]).all()


def test_on_offsets_of_the_path():
    """Offsets and coefficients from the fused FP32 path on the same device,
    fitted with the quality mask, against the oracle's fit of the same
    offsets over the same kept ROIs."""
    from emida_gb300 import GpuOffset, fit_homography, synth as sy
    from oracle import oracle as eo
    ref = sy.reference_pattern(512, seed=61)
    pics, _ = sy.deformed_patterns(512, 61, 3, sigma_eps=3e-3)
    mids, begins = sy.roi_grid(512, 6, 32, margin=40)
    g = GpuOffset((512, 512), begins, (64, 64), (127, 127), 3, "fft", 5, 1, "float", np.uint16, "fused")
    g.allocate_memory(ref)
    offs, coefs = g.get_offset(pics)
    g.close()
    S = len(begins)
    mids = np.asarray(mids, np.float64)
    centre = np.array([256.0, 256.0, 256.0])
    got = fit_homography(mids, offs.reshape(3, S, 2), centre, coefs=coefs.reshape(3, S, 6))
    q = coefs.reshape(3, S, 6)
    keep = (q[..., 3] * q[..., 5] - (q[..., 4] / 2) ** 2) > 1e-6  # det of the negated quadratic
    for k in range(3):
        assert keep[k].sum() > 10
        exp = eo.homography_fit(mids[keep[k]], offs.reshape(3, S, 2)[k][keep[k]], centre)
        assert np.allclose(got[k], exp, rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("scale_exp", [30, -40])
def test_extreme_scales_match_oracle(scale_exp):
    """Coordinates scaled by 2^30 and 2^-40 (exact in FP64): the system's entries scale by
    the square, its column norms leave FP32's range (exponents past +-100), and the
    rotations' zeta is divided in FP64 instead of FP32.  Every entry scales alike, so the
    fitted map is the unscaled one's: both must match the oracle on the unscaled inputs."""
    from emida_gb300 import fit_homography
    from oracle import oracle as eo
    mids, offs, centre = synth(71, 12)
    f = 2.0 ** scale_exp
    got = fit_homography(mids * f, offs * f, centre * f)
    for k in range(len(offs)):
        assert np.allclose(got[k], eo.homography_fit(mids, offs[k], centre), rtol=1e-9, atol=1e-13)
