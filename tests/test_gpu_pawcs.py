"""GPU parity tests of PAWCS (one and three channels): the CUDA path through the C-ABI against the oracle.

Masks, descriptors, every local and global dictionary word, the per-pixel global word tables and all
integer maps must be identical; the FP32 maps (feedback maps, spatial occurrence maps, word weights,
down-sampled averages) must be identical too (tolerance 0 ulp): both sides keep the reference's
operation order without fused multiply-adds. Every compared frame checks the whole model state.
"""
import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorPAWCS, BackgroundSubtractorSuBSENSE, LvException, SyntheticStream, batch_apply
from oracle import pyoracle

pytestmark = pytest.mark.gpu

MAPS = ["R", "V", "T", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST", "ILLUM", "UNSTABLE", "BLINKS",
        "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL", "LAST_RAW_BLINK", "ROI", "LAST_COLOR", "LAST_DESC", "DS_LT", "DS_ST",
        "LUT", "LW_COLOR", "LW_DESC", "LW_OCC", "LW_FIRST", "LW_LAST", "GW", "GW_MAP", "GLUT"]
SCALARS = ["frame_idx", "frames_since_last_reset", "model_reset_cooldown", "lword_weight_offset",
           "auto_model_reset_enabled", "using_moving_camera", "median_blur_kernel_size", "n_local_words",
           "n_global_words", "last_nonflat_ratio", "n_relevant_px", "orig_roi_px", "ds_roi_px"]


def compare_state(gpu, ora):
    bad = []
    for name in MAPS:
        a, b = gpu.state_map(name), ora.state_map(name)
        if a.size != b.size:
            bad.append("%s: %d vs %d bytes" % (name, a.size, b.size))
        elif not np.array_equal(a, b):
            idx = np.flatnonzero(a != b)
            bad.append("%s: %d bytes differ (first at byte %d)" % (name, idx.size, idx[0]))
    sg, so = gpu.scalars(), ora.scalars()
    for k in SCALARS:
        if sg[k] != so[k]:
            bad.append("%s: %r vs %r" % (k, sg[k], so[k]))
    return bad


def run_pair(frames, seed=5, lrs=None, roi=None, check_every=1, **params):
    gpu = BackgroundSubtractorPAWCS(seed=seed, **params)
    ora = pyoracle.OraclePAWCS(seed=seed, **{_oname(k): v for k, v in params.items()})
    gpu.initialize(frames[0], roi)
    ora.initialize(frames[0], roi)
    bad = compare_state(gpu, ora)
    assert not bad, "after initialize: " + "; ".join(bad)
    for t, f in enumerate(frames[1:], start=1):
        lr = 0.0 if lrs is None else lrs[t]
        mg = gpu.apply(f, learningRateOverride=lr)
        mo = ora.apply(f, lr)
        assert np.array_equal(mg, mo), "frame %d: mask differs at %d px" % (t, int((mg != mo).sum()))
        if t % check_every == 0 or t == len(frames) - 1:
            bad = compare_state(gpu, ora)
            assert not bad, "frame %d: %s" % (t, "; ".join(bad))
    return gpu, ora


def _oname(k):
    return {"nDescDistThresholdOffset": "desc_dist_threshold_offset",
            "nMinColorDistThreshold": "min_color_dist_threshold", "nMaxNbWords": "max_words",
            "nSamplesForMovingAvgs": "samples_for_moving_avgs", "fRelLBSPThreshold": "rel_lbsp_threshold"}[k]


def _gray(n, seed, W, H, cfg=0):
    s = SyntheticStream(cfg, 0, seed, width=W, height=H, channels=1)
    return [s.render(t) for t in range(n)]


def test_small_frame_single_global_word():
    # 64x48: one global word (every global item depends on the replaceable word), median 5
    run_pair(_gray(25, 31, 64, 48), seed=3)


def test_moving_shapes_160x120():
    run_pair(_gray(30, 32, 160, 120), seed=4, check_every=3)


def test_thermal_scene_160x120():
    s = SyntheticStream(2, 0, 33, width=160, height=120)
    run_pair([s.render(t) for t in range(30)], seed=5, check_every=3)


def test_full_roi_branch_320x240():
    # frames of 320x240 take the reference's large-frame parameters (median 9, 12 global words,
    # every down-sampled pixel counted)
    s = SyntheticStream(2, 0, 34, width=320, height=240)
    gpu, ora = run_pair([s.render(t) for t in range(17)], seed=6, check_every=8)
    assert gpu.scalars()["median_blur_kernel_size"] == 9


def test_roi_with_border_pixels():
    fr = _gray(20, 35, 96, 72)
    yy, xx = np.mgrid[0:72, 0:96]
    roi = (((xx - 48) / 40.0) ** 2 + ((yy - 36) / 30.0) ** 2 <= 1.0).astype(np.uint8) * 255
    run_pair(fr, seed=7, roi=roi, check_every=4)


def test_learning_rate_overrides():
    fr = _gray(16, 36, 96, 72)
    lrs = [0.0] * 16
    for t in range(4, 8):
        lrs[t] = 1.0
    for t in range(8, 11):
        lrs[t] = float("inf")
    lrs[12] = 3.5
    run_pair(fr, seed=8, lrs=lrs, check_every=2)


def test_automatic_model_reset():
    # a sudden global change of the scene raises the down-sampled L1 ratio above 45 and triggers
    # refreshModel(offset/8, 0, true) with T(x) := 1 and the cool-down
    fr = _gray(26, 37, 96, 72)
    for t in range(14, 26):
        fr[t] = np.clip(fr[t].astype(int) + 120, 0, 255).astype(np.uint8)
    gpu, ora = run_pair(fr, seed=9, check_every=2)
    assert ora.scalars()["model_reset_cooldown"] > 0 or ora.scalars()["frames_since_last_reset"] == 0


def test_refresh_model_and_background_images():
    fr = _gray(14, 38, 96, 72)
    gpu, ora = run_pair(fr[:8], seed=10)
    gpu.refreshModel(5, 0.5, True)
    ora.refresh_model(5, 0.5, True)
    bad = compare_state(gpu, ora)
    assert not bad, "after refreshModel: " + "; ".join(bad)
    for f in fr[8:]:
        assert np.array_equal(gpu.apply(f), ora.apply(f))
    assert not compare_state(gpu, ora)
    assert np.array_equal(gpu.getBackgroundImage(), ora.background())
    assert np.array_equal(gpu.getBackgroundDescriptorsImage(), ora.background_descriptors())


def test_api_errors():
    b = BackgroundSubtractorPAWCS()
    with pytest.raises(LvException):
        b.apply(np.zeros((48, 64), np.uint8))
    with pytest.raises(LvException):
        b.initialize(np.zeros((48, 64, 4), np.uint8))  # four channels: the reference's apply has no such loop
    b.initialize(np.zeros((48, 64), np.uint8))
    with pytest.raises(LvException):
        b.apply(np.zeros((48, 65), np.uint8))
    with pytest.raises(LvException):
        b.refreshModel(1, 1.5)
    with pytest.raises(LvException):
        BackgroundSubtractorPAWCS(nMaxNbWords=1)


def test_config2_full_size_prefix():
    # the benchmark scene itself (640x480 thermal-like), first frames, every mask and the final state
    s = SyntheticStream(2, 0, 1)
    run_pair([s.render(t) for t in range(12)], seed=1, check_every=11)


def test_moving_camera_mode_switch():
    # frames 150-450 darken the scene by 120 levels while an infinite learning-rate override freezes
    # the model: at frame 500 the background image is far from the long-term mean of the down-sampled
    # frames (ratio >= 45 during the bootstrap window), so the moving-camera mode turns on (weight
    # offset 5, refreshModel(1, 1, true)); at frame 1000 the model has caught up and it turns off
    W, H = 64, 48
    s = SyntheticStream(2, 0, 40, width=W, height=H)
    base = [s.render(t).astype(np.int32) for t in range(8)]

    def frame(t):
        return np.clip(base[t % 8] - int(min(max(0, t - 150), 300) * 120 / 300), 0, 255).astype(np.uint8)

    gpu = BackgroundSubtractorPAWCS(seed=11)
    ora = pyoracle.OraclePAWCS(seed=11)
    gpu.initialize(frame(0))
    ora.initialize(frame(0))
    modes = {}
    for t in range(1, 1002):
        lr = float("inf") if 150 <= t <= 500 else 0.0
        mg = gpu.apply(frame(t), learningRateOverride=lr)
        mo = ora.apply(frame(t), lr)
        assert np.array_equal(mg, mo), "frame %d: mask differs at %d px" % (t, int((mg != mo).sum()))
        if t % 100 == 0 or t in (499, 501, 999, 1001):
            bad = compare_state(gpu, ora)
            assert not bad, "frame %d: %s" % (t, "; ".join(bad))
        if t in (499, 500, 999, 1000):
            modes[t] = (gpu.scalars()["using_moving_camera"], gpu.scalars()["lword_weight_offset"])
    assert modes == {499: (0, 1000), 500: (1, 5), 999: (1, 5), 1000: (0, 1000)}


def test_partial_word_rows_72x56():
    # 72 px rows end in a partial bit-plane word (8 bits) in the post-processing kernels
    run_pair(_gray(20, 39, 72, 56), seed=12, check_every=4)


def test_set_roi_reinitializes_from_background():
    fr = _gray(14, 40, 96, 72)
    gpu, ora = BackgroundSubtractorPAWCS(seed=13), pyoracle.OraclePAWCS(seed=13)
    gpu.initialize(fr[0])
    ora.initialize(fr[0])
    for f in fr[1:6]:
        assert np.array_equal(gpu.apply(f), ora.apply(f, 0.0))
    yy, xx = np.mgrid[0:72, 0:96]
    roi = ((((xx - 48) / 40.0) ** 2 + ((yy - 36) / 30.0) ** 2) <= 1.0).astype(np.uint8) * 255
    gpu.setROI(roi)
    ora.set_roi(roi)
    bad = compare_state(gpu, ora)
    assert not bad, "after setROI: " + "; ".join(bad)
    for f in fr[6:]:
        assert np.array_equal(gpu.apply(f), ora.apply(f, 0.0))
    assert not compare_state(gpu, ora)


# ---- three channels (the pixel loop :935-1299: mixed colour distances, neighbour updates that edit the
# target's words) ----

def _bgr(n, seed, W, H, cfg=0):
    s = SyntheticStream(cfg, 0, seed, width=W, height=H, channels=3)
    return [s.render(t) for t in range(n)]


def test_three_channel_small_frame():
    # 64x48: two global words, every frame's whole state
    run_pair(_bgr(20, 51, 64, 48), seed=6)


def test_three_channel_moving_shapes_160x120():
    run_pair(_bgr(30, 52, 160, 120), seed=7, check_every=3)


def test_three_channel_lr_schedule_roi_and_background():
    # the application's schedule (learning rate 1 for the first frames), an elliptic ROI, then
    # refreshModel and the background images
    fr = _bgr(18, 53, 96, 72)
    yy, xx = np.mgrid[0:72, 0:96]
    roi = ((((xx - 48) / 44.0) ** 2 + ((yy - 36) / 32.0) ** 2) <= 1.0).astype(np.uint8) * 255
    lrs = [1.0 if t <= 6 else 0.0 for t in range(12)]
    gpu, ora = run_pair(fr[:12], seed=14, lrs=lrs, roi=roi, check_every=2)
    gpu.refreshModel(3, 0.25, True)
    ora.refresh_model(3, 0.25, True)
    bad = compare_state(gpu, ora)
    assert not bad, "after refreshModel: " + "; ".join(bad)
    for f in fr[12:]:
        assert np.array_equal(gpu.apply(f), ora.apply(f))
    assert not compare_state(gpu, ora)
    assert np.array_equal(gpu.getBackgroundImage(), ora.background())
    assert np.array_equal(gpu.getBackgroundDescriptorsImage(), ora.background_descriptors())


def test_three_channel_fixed_point_rounds_and_partial_words():
    # 72 px rows (partial bit-plane words); the earlier updaters' word edits need more than one round
    gpu, ora = run_pair(_bgr(16, 54, 72, 56), seed=15, check_every=3)
    rounds = []
    s = SyntheticStream(0, 0, 55, width=72, height=56, channels=3)
    g2 = BackgroundSubtractorPAWCS(seed=16)
    g2.initialize(s.render(0))
    for t in range(1, 8):
        g2.apply(s.render(t))
        rounds.append(g2.scalars()["fixed_point_rounds"])
    assert max(rounds) >= 2, rounds


def test_three_channel_full_size_prefix():
    # a 640x480 BGR scene: the three-channel geometry at full size (50 local, 25 global words, median 13)
    s = SyntheticStream(0, 0, 56, width=640, height=480, channels=3)
    gpu, ora = run_pair([s.render(t) for t in range(6)], seed=17, check_every=5)
    sc = gpu.scalars()
    assert (sc["n_local_words"], sc["n_global_words"]) == (50, 25)


def test_three_channel_moving_camera_mode_switch():
    # as the one-channel case, on BGR frames: the camera-motion comparison adds the colour distortion
    # ratio of the down-sampled background image (lv::cdist on floats)
    W, H = 64, 48
    s = SyntheticStream(0, 0, 57, width=W, height=H, channels=3)
    base = [s.render(t).astype(np.int32) for t in range(8)]

    def frame(t):
        return np.clip(base[t % 8] - int(min(max(0, t - 150), 300) * 120 / 300), 0, 255).astype(np.uint8)

    gpu = BackgroundSubtractorPAWCS(seed=18)
    ora = pyoracle.OraclePAWCS(seed=18)
    gpu.initialize(frame(0))
    ora.initialize(frame(0))
    modes = {}
    for t in range(1, 1002):
        lr = float("inf") if 150 <= t <= 500 else 0.0
        mg = gpu.apply(frame(t), learningRateOverride=lr)
        mo = ora.apply(frame(t), lr)
        assert np.array_equal(mg, mo), "frame %d: mask differs at %d px" % (t, int((mg != mo).sum()))
        if t % 100 == 0 or t in (499, 501, 999, 1001):
            bad = compare_state(gpu, ora)
            assert not bad, "frame %d: %s" % (t, "; ".join(bad))
        if t in (499, 500, 999, 1000):
            modes[t] = gpu.scalars()["using_moving_camera"]
    assert modes[499] == 0 and modes[500] == 1, modes


def test_three_channel_set_roi_reinitializes_from_background():
    # setROI re-initializes from the three-channel background image with the new ROI
    fr = _bgr(14, 58, 96, 72)
    gpu, ora = BackgroundSubtractorPAWCS(seed=19), pyoracle.OraclePAWCS(seed=19)
    gpu.initialize(fr[0])
    ora.initialize(fr[0])
    for f in fr[1:6]:
        assert np.array_equal(gpu.apply(f), ora.apply(f, 0.0))
    yy, xx = np.mgrid[0:72, 0:96]
    roi = ((((xx - 48) / 40.0) ** 2 + ((yy - 36) / 30.0) ** 2) <= 1.0).astype(np.uint8) * 255
    gpu.setROI(roi)
    ora.set_roi(roi)
    bad = compare_state(gpu, ora)
    assert not bad, "after setROI: " + "; ".join(bad)
    for f in fr[6:]:
        assert np.array_equal(gpu.apply(f), ora.apply(f, 0.0))
    assert not compare_state(gpu, ora)


@pytest.mark.parametrize("W,H,C", [(595, 245, 1), (640, 350, 3)])
def test_non_integral_down_sampling(W, H, C):
    """Sizes whose 1/8 down-sampling is not integral: INTER_AREA of the ROI (:446) and of each frame
    (:1475) as the exact area-weighted mean."""
    s = SyntheticStream(0, 0, 43, width=W, height=H, channels=C)
    run_pair([s.render(t) for t in range(8)], seed=15, check_every=2)


@pytest.mark.parametrize("channels", [1, 3])
def test_spill_restore_is_transparent(channels):
    """lvbgs_spill / lvbgs_restore of a PAWCS stream: the model evolves bit-identically across the pair
    (every mask and, at the end, every map equal to the oracle's)."""
    s = SyntheticStream(0, 0, 44, width=128, height=96, channels=channels)
    frames = [s.render(t) for t in range(14)]
    a = BackgroundSubtractorPAWCS(seed=3)
    ora = pyoracle.OraclePAWCS(seed=3)
    a.initialize(frames[0])
    ora.initialize(frames[0])
    for t in range(1, 14):
        if t in (5, 9):
            buf = bytearray(a.state_bytes())
            a.spill(buf)
            with pytest.raises(LvException):
                a.apply(frames[t])
            a.restore(buf)
        assert np.array_equal(a.apply(frames[t]), ora.apply(frames[t])), "frame %d" % t
    bad = compare_state(a, ora)
    assert not bad, "; ".join(bad)


@pytest.mark.parametrize("with_subsense", [False, True])
def test_batched_pawcs_streams_equal_streams_alone(with_subsense):
    """lvbgs_batch_apply with PAWCS streams (one BGR, one gray), alone or beside a SuBSENSE stream: the
    PAWCS steps run in flight together on their handles' own streams and the SuBSENSE one as a batched
    step; every mask equals the oracle's stream run alone, also across a spill / restore of a PAWCS
    stream between two batches, and the PAWCS models end identical to the oracle's."""
    sp = [SyntheticStream(0, 0, 51, width=128, height=96, channels=3), SyntheticStream(0, 0, 52, width=96, height=64,
                                                                                       channels=1)]
    fp = [[s.render(t) for t in range(12)] for s in sp]
    pw = [BackgroundSubtractorPAWCS(seed=7), BackgroundSubtractorPAWCS(seed=8)]
    opw = [pyoracle.OraclePAWCS(seed=7), pyoracle.OraclePAWCS(seed=8)]
    for g, o, f in zip(pw, opw, fp):
        g.initialize(f[0])
        o.initialize(f[0])
    subs, osub, fs = [], [], []
    if with_subsense:
        ss = SyntheticStream(0, 0, 53, width=160, height=120, channels=3)
        fs = [ss.render(t) for t in range(12)]
        subs = [BackgroundSubtractorSuBSENSE(seed=9)]
        osub = [pyoracle.OracleSuBSENSE(seed=9)]
        subs[0].initialize(fs[0])
        osub[0].initialize(fs[0])
    for t in range(1, 12):
        if t == 6:
            buf = bytearray(pw[0].state_bytes())
            pw[0].spill(buf)
            pw[0].restore(buf)
        handles = [pw[0]] + subs + [pw[1]]
        images = [fp[0][t]] + [f[t] for f in ([fs] if subs else [])] + [fp[1][t]]
        masks = batch_apply(handles, images)
        want = [opw[0].apply(fp[0][t])] + [o.apply(fs[t]) for o in osub] + [opw[1].apply(fp[1][t])]
        for i, (m, w) in enumerate(zip(masks, want)):
            assert np.array_equal(m, w), "frame %d, batch entry %d: mask differs at %d px" % (t, i, int((m != w).sum()))
    for g, o in zip(pw, opw):
        bad = compare_state(g, o)
        assert not bad, "; ".join(bad)
