"""CPU tests of the PAWCS oracle (oracle/pawcs.c): the geometry-dependent parameters of
BackgroundSubtractorPAWCS::initialize (BackgroundSubtractorPAWCS.cpp:446-466), model invariants,
determinism, segmentation sanity on the thermal-like scene, and input checks."""
import numpy as np
import pytest

from litiv_gb300.synth import SyntheticStream
from oracle import pyoracle


def _frames(n, seed=3, **over):
    s = SyntheticStream(2, 0, seed, **over)
    return s, [s.render(t) for t in range(n)]


def test_config2_geometry_parameters():
    # 640x480 gray, full ROI: median 13, 50/2 = 25 local and 25/2 = 12 global words, all 80x60
    # down-sampled pixels count for the frame-level analysis (|= 127)
    img = SyntheticStream(2, 0, 1).render(0)
    o = pyoracle.OraclePAWCS(seed=1)
    o.initialize(img)
    s = o.scalars()
    assert (s["median_blur_kernel_size"], s["n_local_words"], s["n_global_words"]) == (13, 25, 12)
    assert s["ds_roi_px"] == 80 * 60
    assert s["n_relevant_px"] == 636 * 476 and s["orig_roi_px"] == 640 * 480
    assert s["auto_model_reset_enabled"] == 1 and s["lword_weight_offset"] == 1000


def test_small_color_frame_parameters():
    # 160x120 BGR (< 320x240): G = min((size_t)pow(25 * 0.25, 2) + 1, 25) = 25, median
    # min(floor(0.5 + 9 * 0.25 * 2) + 5, 9) = 9; three channels keep 50 local words
    img = SyntheticStream(0, 0, 2, width=160, height=120, channels=3).render(0)
    o = pyoracle.OraclePAWCS(seed=2)
    o.initialize(img)
    s = o.scalars()
    assert (s["median_blur_kernel_size"], s["n_local_words"], s["n_global_words"]) == (9, 50, 25)


@pytest.mark.parametrize("channels", [1, 3])
def test_model_invariants_after_initialize(channels):
    img = SyntheticStream(0, 0, 4, width=96, height=64, channels=channels).render(0)
    o = pyoracle.OraclePAWCS(seed=4)
    o.initialize(img)
    s = o.scalars()
    L, G = s["n_local_words"], s["n_global_words"]
    occ = o.state_map("LW_OCC").view(np.uint64)
    assert occ.size == s["n_relevant_px"] * L and (occ > 0).all()
    first = o.state_map("LW_FIRST").view(np.uint64)
    assert (first == 0).all()
    glut = o.state_map("GLUT").reshape(64 * 96, G)
    roi = o.state_map("ROI").reshape(64, 96)
    rows = glut[roi.ravel() > 0]
    assert (np.sort(rows, axis=1) == np.arange(G)).all()  # every per-pixel table is a permutation
    gw = o.state_map("GW").reshape(G, 20)
    slots = gw[:, 16:20].copy().view(np.int32).ravel()
    assert sorted(slots.tolist()) == list(range(G))  # every pool word sits in one dictionary slot


def test_deterministic_and_seeded():
    _, fr = _frames(12, width=128, height=96)
    masks = []
    for seed in (9, 9, 10):
        o = pyoracle.OraclePAWCS(seed=seed)
        o.initialize(fr[0])
        masks.append([o.apply(f) for f in fr[1:]])
    assert all(np.array_equal(a, b) for a, b in zip(masks[0], masks[1]))
    o9 = pyoracle.OraclePAWCS(seed=9)
    o10 = pyoracle.OraclePAWCS(seed=10)
    o9.initialize(fr[0])
    o10.initialize(fr[0])
    assert not np.array_equal(o9.state_map("LW_COLOR"), o10.state_map("LW_COLOR"))


@pytest.mark.parametrize("channels", [1, 3])
def test_moving_shapes_are_segmented(channels):
    s = SyntheticStream(0, 0, 3 + channels, width=160, height=120, channels=channels)
    fr = [s.render(t) for t in range(40)]
    o = pyoracle.OraclePAWCS(seed=5)
    o.initialize(fr[0])
    for f in fr[1:]:
        m = o.apply(f)
    gt = s.render(39, with_gt=True)[1] > 0
    fg = m > 0
    assert gt.sum() > 0
    assert (fg & gt).sum() / gt.sum() > 0.5
    assert (fg & ~gt).sum() / max(1, (~gt).sum()) < 0.1


def test_thermal_scene_runs():
    # blobs that move away from where the model first saw them show up as foreground
    s, fr = _frames(21, seed=5, width=320, height=240)
    o = pyoracle.OraclePAWCS(seed=5)
    o.initialize(fr[0])
    for f in fr[1:]:
        m = o.apply(f)
    moved = (s.render(20, with_gt=True)[1] > 0) & ~(s.render(0, with_gt=True)[1] > 0)
    assert (m > 0).any() and ((m > 0) & moved).any()


def test_background_image_of_a_static_scene():
    s = SyntheticStream(2, 0, 6, width=96, height=64, n_shapes=0)
    fr = [s.render(t) for t in range(6)]
    o = pyoracle.OraclePAWCS(seed=6)
    o.initialize(fr[0])
    for f in fr[1:]:
        o.apply(f)
    bg = o.background().astype(int)
    inner = (slice(2, -2), slice(2, -2))
    assert np.abs(bg[inner] - fr[-1].astype(int)[inner]).mean() < 6
    d = o.background_descriptors()
    assert d.dtype == np.uint16 and d.shape == (64, 96)


def test_input_checks():
    o = pyoracle.OraclePAWCS(seed=1)
    img = np.zeros((48, 64), np.uint8)
    with pytest.raises(ValueError):
        o.initialize(img, roi=np.full((48, 64), 7, np.uint8))  # ROI must be 0/255
    with pytest.raises(ValueError):
        o.initialize(np.zeros((48, 64, 2), np.uint8))
    o.initialize(img)
    assert o.refresh_model(1, 1.5) != 0  # occurrence decrement fraction must be in [0, 1]
    assert o.refresh_model(1, 0.5, force=True) == 0
    with pytest.raises(ValueError):
        pyoracle.OraclePAWCS(seed=1, max_words=1)  # max/2 global words must be positive
