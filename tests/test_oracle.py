"""CPU tests of the oracle: pinned by the reference's golden vector and its property tests."""
import os

import numpy as np
import pytest

from oracle import pyoracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# Random123 known-answer vectors for Philox4x32-10 (ctr, key, expected)
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


def lbsp_numpy(img, thr_fn):
    """Direct restatement of LBSP.hpp:297-319 for cross-checking (bit n = |tap_n - ref| > thr)."""
    dx = [-2, 2, 0, 0, -2, 2, 2, -2, 0, -1, 0, 1, -1, 1, 1, -1]
    dy = [0, 0, -2, 2, 2, -2, 2, -2, 1, 0, -1, 0, -1, 1, -1, 1]
    im = img.astype(np.int32)
    if im.ndim == 2:
        im = im[:, :, None]
    H, W, C = im.shape
    out = np.zeros((H, W, C), np.uint16)
    ref = im[2:H - 2, 2:W - 2]
    thr = thr_fn(ref)
    acc = np.zeros(ref.shape, np.int32)
    for n in range(16):
        tap = im[2 + dy[n]:H - 2 + dy[n], 2 + dx[n]:W - 2 + dx[n]]
        acc |= (np.abs(tap - ref) > thr).astype(np.int32) << n
    out[2:H - 2, 2:W - 2] = acc
    return out if img.ndim == 3 else out[:, :, 0]


def test_philox_known_answers(oracle_lib):
    for ctr, key, exp in PHILOX_KAT:
        assert pyoracle.philox(ctr, key) == exp


def test_lbsp_golden_vector(oracle_lib):
    """lbsp.regression_compute (modules/features2d/test/lbsp.cpp:22-46): LBSP(20) on the 65x65 crop,
    compared on the inner 61x61 zone against test_lbsp.bin."""
    img = np.load(os.path.join(GOLDEN, "lbsp_input_65x65_bgr.npy"))
    gold = np.load(os.path.join(GOLDEN, "lbsp_abs20_65x65_u16c3.npy"))
    desc = pyoracle.lbsp_compute2(img, abs_threshold=20)
    np.testing.assert_array_equal(desc[2:-2, 2:-2], gold[2:-2, 2:-2])


@pytest.mark.parametrize("channels", [1, 3])
def test_lbsp_relative_threshold_matches_restatement(oracle_lib, channels):
    rng = np.random.default_rng(3)
    shape = (37, 41, channels) if channels == 3 else (37, 41)
    img = rng.integers(0, 256, shape, dtype=np.uint8)
    desc = pyoracle.lbsp_compute2(img, abs_threshold=None, rel_threshold=0.333, offset=0)

    def thr(ref):
        # saturate_cast<uchar>(ref*0.333f + 0) with round half to even, in float
        return np.clip(np.rint((ref.astype(np.float32) * np.float32(0.333)).astype(np.float32)), 0, 255)

    ref = lbsp_numpy(img, thr)
    np.testing.assert_array_equal(desc[2:-2, 2:-2], ref[2:-2, 2:-2])


def test_sample_position_7x7_weights_and_bounds(oracle_lib):
    """getSamplePosition_7x7_std2 (opencv.hpp:909-925): r = 1 + rand%512 walks the 7x7 weights, so
    the 512 residues hit each offset exactly `weight` times; positions are clamped to the border."""
    import ctypes as C
    L = oracle_lib
    weights = np.array([[2, 4, 6, 7, 6, 4, 2], [4, 8, 12, 14, 12, 8, 4], [6, 12, 21, 25, 21, 12, 6],
                        [7, 14, 25, 28, 25, 14, 7], [6, 12, 21, 25, 21, 12, 6], [4, 8, 12, 14, 12, 8, 4],
                        [2, 4, 6, 7, 6, 4, 2]])
    counts = np.zeros((7, 7), int)
    sx, sy = C.c_int(), C.c_int()
    for r in range(512):
        L.osample_pos_7x7(r + 512 * 12345, 100, 80, 640, 480, C.byref(sx), C.byref(sy))
        counts[sy.value - 80 + 3, sx.value - 100 + 3] += 1
    np.testing.assert_array_equal(counts, weights)
    for r in range(0, 2 ** 31 - 1, 2 ** 21 + 17):
        L.osample_pos_7x7(r, 0, 0, 640, 480, C.byref(sx), C.byref(sy))
        assert 2 <= sx.value <= 3 and 2 <= sy.value <= 3
        L.osample_pos_7x7(r, 639, 479, 640, 480, C.byref(sx), C.byref(sy))
        assert 636 <= sx.value <= 637 and 476 <= sy.value <= 477


@pytest.mark.parametrize("use3x3,radius,count", [(1, 1, 8), (0, 2, 24)])
def test_neighbor_position_properties(oracle_lib, use3x3, radius, count):
    """getNeighborPosition.regression (utils/test/opencv.cpp:416-429): within the window, never the
    centre away from the border, every neighbour reachable."""
    import ctypes as C
    nx, ny = C.c_int(), C.c_int()
    seen = set()
    rng = np.random.default_rng(5)
    for r in rng.integers(0, 2 ** 31 - 1, 5000):
        oracle_lib.oneighbor_pos(int(r), use3x3, 320, 240, 640, 480, C.byref(nx), C.byref(ny))
        assert abs(nx.value - 320) <= radius and abs(ny.value - 240) <= radius
        assert not (nx.value == 320 and ny.value == 240)
        seen.add((nx.value, ny.value))
    assert len(seen) == count
    oracle_lib.oneighbor_pos(0, use3x3, 2, 2, 640, 480, C.byref(nx), C.byref(ny))
    assert nx.value >= 2 and ny.value >= 2


def _fmeasure(mask, gt):
    tp = np.sum((mask > 0) & (gt > 0))
    fp = np.sum((mask > 0) & (gt == 0))
    fn = np.sum((mask == 0) & (gt > 0))
    return 2 * tp / max(1, 2 * tp + fp + fn)


def test_oracle_segments_synthetic_scene(product_lib):
    from litiv_gb300 import SyntheticStream
    s = SyntheticStream(0, seed=2)
    o = pyoracle.OracleSuBSENSE(seed=11)
    o.initialize(s.render(0))
    fms = []
    for t in range(1, 41):
        f, g = s.render(t, with_gt=True)
        m = o.apply(f)
        assert set(np.unique(m)) <= {0, 255}
        if t > 15:
            fms.append(_fmeasure(m, g))
    assert np.mean(fms) > 0.4
    sc = o.scalars()
    assert sc["frame_idx"] == 40 and sc["median_blur_kernel_size"] == 9 and sc["use_3x3_spread"] == 1


def test_oracle_deterministic_and_seeded(product_lib):
    from litiv_gb300 import SyntheticStream
    s = SyntheticStream(0, seed=4)
    frames = [s.render(t) for t in range(8)]
    runs = []
    for seed in (1, 1, 2):
        o = pyoracle.OracleSuBSENSE(seed=seed)
        o.initialize(frames[0])
        runs.append([o.apply(f) for f in frames[1:]] + [o.state_map("SAMPLE_COLOR").copy()])
    for a, b in zip(runs[0], runs[1]):
        np.testing.assert_array_equal(a, b)
    assert not np.array_equal(runs[0][-1], runs[2][-1])


def test_oracle_argument_errors(oracle_lib):
    with pytest.raises(ValueError):
        pyoracle.OracleSuBSENSE(required_bg_samples=60)
    with pytest.raises(ValueError):
        pyoracle.OracleSuBSENSE(min_color_dist_threshold=0, desc_dist_threshold_offset=0)
    o = pyoracle.OracleSuBSENSE()
    img = np.zeros((20, 20, 3), np.uint8)
    with pytest.raises(ValueError):
        o.initialize(img, roi=np.full((20, 20), 7, np.uint8))  # ROI values must be 0/255
    with pytest.raises(ValueError):
        o.initialize(img, roi=np.zeros((20, 20), np.uint8))  # no useful pixels
    with pytest.raises(ValueError):
        o.initialize(np.zeros((20, 20, 4), np.uint8))  # 8UC4 has no apply() loop
    assert o.refresh_model(0.5) != 0  # not initialized


def test_oracle_roi_excludes_pixels(product_lib):
    from litiv_gb300 import SyntheticStream
    s = SyntheticStream(0, seed=6)
    roi = np.zeros((240, 320), np.uint8)
    roi[40:200, 60:260] = 255
    o = pyoracle.OracleSuBSENSE(seed=3)
    o.initialize(s.render(0), roi)
    r = o.state_map("ROI")
    assert r[40, 60] == 255 and r[0, 0] == 0 and r[39, 60] == 128  # 255/2 rounded half to even near the ROI edge
    for t in range(1, 6):
        o.apply(s.render(t))
    raw = o.state_map("LAST_RAW_FG")
    assert raw[r == 0].max() == 0


def test_oracle_roi_rules():
    # setROI before initialize keeps the validated ROI as is; initialize() without a ROI of the same size
    # reuses the last validated ROI; setROI on an initialized model re-initializes (edge pixels 128)
    from litiv_gb300 import SyntheticStream
    s = SyntheticStream(0, seed=63, width=96, height=72, shape_min=10, shape_max=24)
    fr = [s.render(t) for t in range(3)]
    yy, xx = np.mgrid[0:72, 0:96]
    roi = ((((xx - 48) / 40.0) ** 2 + ((yy - 36) / 30.0) ** 2) <= 1.0).astype(np.uint8) * 255
    v = roi.copy()
    v[:2] = 0
    v[-2:] = 0
    v[:, :2] = 0
    v[:, -2:] = 0
    o = pyoracle.OracleSuBSENSE(seed=1)
    o.set_roi(roi)
    o.initialize(fr[0])
    assert np.array_equal(o.state_map("ROI"), v)
    o.apply(fr[1], 0.0)
    o.initialize(fr[2])
    assert np.array_equal(o.state_map("ROI"), v)
    o.set_roi(roi)
    assert set(np.unique(o.state_map("ROI")).tolist()) == {0, 128, 255}
