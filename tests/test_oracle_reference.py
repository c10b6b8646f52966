"""CPU tests that pin the C restatement (oracle/subsense.c, oracle/pawcs.c, oracle/lobster.c) to the
REFERENCE itself.

oracle/_ref/libref.so is the reference's own BackgroundSubtractorSuBSENSE / BackgroundSubtractorPAWCS /
BackgroundSubtractorLOBSTER / BackgroundSubtractorLBSP / BackgroundSubtractionUtils sources
(modules/video/src), compiled unmodified
against a project-written OpenCV stand-in with rand() routed to the counter-based generator
(oracle/refshim/build_ref.py). Both run on the same frames and every model map is compared after
initialize() and after every frame: masks, every integer map, every FP32 map (tolerance 0 ulp), all
samples / local and global words, the LBSP threshold LUT and the frame-level scalars. The GPU parity
tests compare the GPU with the restatement, so together they pin the GPU to the reference.

The reference sources are read where they lie, so these tests run only where they are present
(skipped elsewhere, e.g. on a machine that only has this repository).
"""
import numpy as np
import pytest

from oracle import pyoracle
from oracle.pyoracle import MAP_NAMES, PAWCS_MAP_NAMES

if pyoracle.ref_lib() is None:
    pytest.skip("the reference sources are not present here", allow_module_level=True)

# scalars that are per-frame counters of the restatement only (the reference keeps them local)
_PORT_ONLY = ("stat_", "nonzero_desc_count", "tot_color_diff")


def _frames(config, n, seed, **kw):
    from litiv_gb300 import SyntheticStream
    s = SyntheticStream(config, 0, seed, **kw)
    return [s.render(t) for t in range(n)]


def _compare(port, ref, names, where):
    for nm in names:
        a = np.asarray(port.state_map(nm)).view(np.uint8).ravel()
        b = np.asarray(ref.state_map(nm)).view(np.uint8).ravel()
        assert a.shape == b.shape, "%s: %s sizes differ (%s vs %s)" % (where, nm, a.shape, b.shape)
        if not np.array_equal(a, b):
            raise AssertionError("%s: %s differs in %d bytes" % (where, nm, int((a != b).sum())))
    sp, sr = port.scalars(), ref.scalars()
    diff = {k: (sp[k], sr[k]) for k in sp if not k.startswith(_PORT_ONLY) and sp[k] != sr[k]}
    assert not diff, "%s: scalars differ %s" % (where, diff)


def run_both(cls, names, frames, seed, lrs=None, roi=None, check_every=1, **params):
    port = cls(seed=seed, impl="port", **params)
    ref = cls(seed=seed, impl="reference", **params)
    port.initialize(frames[0], roi)
    ref.initialize(frames[0], roi)
    _compare(port, ref, names, "after initialize")
    for t, f in enumerate(frames[1:], start=1):
        lr = 0.0 if lrs is None else lrs[t]
        mp, mr = port.apply(f, lr), ref.apply(f, lr)
        assert np.array_equal(mp, mr), "frame %d: mask differs at %d px" % (t, int((mp != mr).sum()))
        if t % check_every == 0 or t == len(frames) - 1:
            _compare(port, ref, names, "frame %d" % t)
    return port, ref


def sub_pair(frames, seed, **kw):
    return run_both(pyoracle.OracleSuBSENSE, MAP_NAMES, frames, seed, **kw)


def pawcs_pair(frames, seed, **kw):
    return run_both(pyoracle.OraclePAWCS, PAWCS_MAP_NAMES, frames, seed, **kw)


# ---------------- SuBSENSE (modules/video/src/BackgroundSubtractorSuBSENSE.cpp) ----------------

def test_subsense_config0_scene_40_frames():
    """320x240 BGR (the config 0 scene): includes the three-channel last-distance term whose colour
    L1 wraps modulo 256 in the reference (lv::L1dist<3> accumulates in unsigned char)."""
    sub_pair(_frames(0, 41, 1), seed=1)


def test_subsense_gray():
    sub_pair(_frames(0, 31, 8, channels=1), seed=2, check_every=3)


def test_subsense_small_frame_without_frame_level_analysis():
    sub_pair(_frames(0, 25, 3, width=48, height=40, shape_min=6, shape_max=14), seed=9)


def test_subsense_learning_rate_schedule():
    frames = _frames(0, 31, 4, width=96, height=72, shape_min=10, shape_max=24)
    sub_pair(frames, seed=4, lrs=[1.0 if t <= 20 else 0.0 for t in range(31)])


def test_subsense_roi():
    roi = np.zeros((240, 320), np.uint8)
    roi[30:210, 50:270] = 255
    roi[100:140, 120:200] = 0
    sub_pair(_frames(0, 21, 6), seed=6, roi=roi, check_every=4)


def test_subsense_automatic_model_reset():
    frames = _frames(0, 48, 12)
    for t in range(30, 48):
        frames[t] = np.clip(frames[t].astype(np.int16) + 150, 0, 255).astype(np.uint8)
    port, ref = sub_pair(frames, seed=12, check_every=2)
    assert ref.scalars()["model_reset_cooldown"] > 0  # the reset fired


def test_subsense_1080p_prefix():
    """1920x1080 BGR (the config 1 scene): 13x13 median, 5x5 neighbour spread, frame-level analysis."""
    port, ref = sub_pair(_frames(1, 3, 1), seed=1)
    assert ref.scalars()["median_blur_kernel_size"] == 13 and ref.scalars()["use_3x3_spread"] == 0


def test_subsense_set_roi_refresh_and_background_images():
    frames = _frames(0, 14, 20, width=96, height=72, shape_min=8, shape_max=20)
    port, ref = sub_pair(frames[:6], seed=20)
    port.refresh_model(0.3, True)
    ref.refresh_model(0.3, True)
    _compare(port, ref, MAP_NAMES, "after refreshModel")
    assert np.array_equal(port.background(), ref.background())
    assert np.array_equal(port.background_descriptors(), ref.background_descriptors())
    yy, xx = np.mgrid[0:72, 0:96]
    roi = ((((xx - 48) / 40.0) ** 2 + ((yy - 36) / 30.0) ** 2) <= 1.0).astype(np.uint8) * 255
    port.set_roi(roi)
    ref.set_roi(roi)
    _compare(port, ref, MAP_NAMES, "after setROI")
    for t, f in enumerate(frames[6:], start=6):
        assert np.array_equal(port.apply(f), ref.apply(f)), "frame %d" % t
    _compare(port, ref, MAP_NAMES, "end")


# ---------------- PAWCS (modules/video/src/BackgroundSubtractorPAWCS.cpp) ----------------

def test_pawcs_config2_scene_prefix():
    """640x480 single-channel thermal-like scene (config 2)."""
    pawcs_pair(_frames(2, 9, 1), seed=1, check_every=4)


def test_pawcs_single_channel_moving_shapes():
    pawcs_pair(_frames(0, 30, 32, width=160, height=120, channels=1), seed=4, check_every=3)


def test_pawcs_three_channels():
    """Three channels: every colour L1 and cmixdist of the reference wraps modulo 256."""
    pawcs_pair(_frames(0, 30, 11, width=160, height=120), seed=5, check_every=3)


@pytest.mark.parametrize("channels", [1, 3])
def test_pawcs_roi_and_learning_rate_overrides(channels):
    fr = _frames(0, 16, 36, width=96, height=72, channels=channels)
    yy, xx = np.mgrid[0:72, 0:96]
    roi = (((xx - 48) / 40.0) ** 2 + ((yy - 36) / 30.0) ** 2 <= 1.0).astype(np.uint8) * 255
    lrs = [0.0] * 16
    for t in range(4, 8):
        lrs[t] = 1.0
    for t in range(8, 11):
        lrs[t] = float("inf")
    lrs[12] = 3.5
    pawcs_pair(fr, seed=8, roi=roi, lrs=lrs, check_every=2)


def test_pawcs_automatic_model_reset():
    fr = _frames(0, 26, 37, width=96, height=72, channels=1)
    for t in range(14, 26):
        fr[t] = np.clip(fr[t].astype(int) + 120, 0, 255).astype(np.uint8)
    pawcs_pair(fr, seed=9, check_every=2)


@pytest.mark.parametrize("channels", [1, 3])
def test_pawcs_refresh_model_and_background_images(channels):
    fr = _frames(0, 12, 38, width=96, height=72, channels=channels)
    port, ref = pawcs_pair(fr[:7], seed=10)
    port.refresh_model(5, 0.5, True)
    ref.refresh_model(5, 0.5, True)
    _compare(port, ref, PAWCS_MAP_NAMES, "after refreshModel")
    for f in fr[7:]:
        assert np.array_equal(port.apply(f), ref.apply(f))
    _compare(port, ref, PAWCS_MAP_NAMES, "end")
    assert np.array_equal(port.background(), ref.background())
    assert np.array_equal(port.background_descriptors(), ref.background_descriptors())


def test_pawcs_moving_camera_mode_switch():
    """Camera-motion check every 500 frames (:1478-1499): the mode turns on at 500, off at 1000."""
    W, H = 64, 48
    from litiv_gb300 import SyntheticStream
    s = SyntheticStream(2, 0, 40, width=W, height=H)
    base = [s.render(t).astype(np.int32) for t in range(8)]

    def frame(t):
        return np.clip(base[t % 8] - int(min(max(0, t - 150), 300) * 120 / 300), 0, 255).astype(np.uint8)

    port = pyoracle.OraclePAWCS(seed=11, impl="port")
    ref = pyoracle.OraclePAWCS(seed=11, impl="reference")
    port.initialize(frame(0))
    ref.initialize(frame(0))
    modes = {}
    for t in range(1, 1002):
        lr = float("inf") if 150 <= t <= 500 else 0.0
        assert np.array_equal(port.apply(frame(t), lr), ref.apply(frame(t), lr)), "frame %d" % t
        if t % 250 == 0 or t in (501, 1001):
            _compare(port, ref, PAWCS_MAP_NAMES, "frame %d" % t)
        if t in (499, 500, 999, 1000):
            modes[t] = ref.scalars()["using_moving_camera"]
    assert modes == {499: 0, 500: 1, 999: 1, 1000: 0}


@pytest.mark.parametrize("algo,shape", [("subsense", (350, 640, 3)), ("subsense", (245, 595, 3)),
                                        ("pawcs", (245, 595, 1)), ("pawcs", (350, 640, 3))])
def test_non_integral_frame_level_down_sampling(algo, shape):
    """Frame sizes whose 1/8 down-sampling is not integral (common CDnet sizes): INTER_AREA with a
    non-integral scale in the frame-level analysis (BackgroundSubtractorSuBSENSE.cpp:568,
    BackgroundSubtractorPAWCS.cpp:446,1475)."""
    H, W, C = shape
    frames = _frames(0, 8, 41, width=W, height=H, channels=C)
    pair = sub_pair if algo == "subsense" else pawcs_pair
    pair(frames, seed=13, check_every=2)


# ---- LOBSTER (BackgroundSubtractorLOBSTER.cpp:410-620) ----
LOB_NAMES = pyoracle.LOBSTER_MAP_NAMES


def _lob_run(frames, seed, lrs=None, roi=None, refreshes=(), **params):
    """run_both for LOBSTER (its learning rate is an integer-like rate > 0, default 16); refreshes:
    (frame index, fraction, force) refreshModel calls made after that frame"""
    port = pyoracle.OracleLOBSTER(seed=seed, impl="port", **params)
    ref = pyoracle.OracleLOBSTER(seed=seed, impl="reference", **params)
    port.initialize(frames[0], roi)
    ref.initialize(frames[0], roi)
    _compare(port, ref, LOB_NAMES, "after initialize")
    for t, f in enumerate(frames[1:], start=1):
        lr = 16.0 if lrs is None else lrs[t]
        mp, mr = port.apply(f, lr), ref.apply(f, lr)
        assert np.array_equal(mp, mr), "frame %d: mask differs at %d px" % (t, int((mp != mr).sum()))
        _compare(port, ref, LOB_NAMES, "frame %d" % t)
        for (ti, frac, force) in refreshes:
            if ti == t:
                assert port.refresh_model(frac, force) == 0 and ref.refresh_model(frac, force) == 0
                _compare(port, ref, LOB_NAMES, "refresh after frame %d" % t)
    return port, ref


@pytest.mark.parametrize("config", [0, 2])
def test_lobster_scene(config):
    # config 0: 320x240 BGR moving shapes; config 2: 640x480 single-channel scene
    _lob_run(_frames(config, 16, 1), seed=21)


def test_lobster_learning_rates_roi_refresh_and_background_images():
    fr = _frames(0, 14, 3)
    roi = np.zeros(fr[0].shape[:2], np.uint8)
    roi[20:200, 30:290] = 255
    lrs = [16.0, 1.0, 1.0, 2.0, 3.5, 16.0, float("inf"), 1.0, 4.0, 16.0, 1.0, 2.0, 16.0, 1.0]
    port, ref = _lob_run(fr, seed=4, lrs=lrs, roi=roi, refreshes=((5, 0.4, False), (9, 1.0, True)))
    assert np.array_equal(port.background(), ref.background())
    assert np.array_equal(port.background_descriptors(), ref.background_descriptors())


def test_lobster_parameters_gray():
    fr = _frames(0, 10, 5, channels=1)
    _lob_run(fr, seed=8, bg_samples=20, required_bg_samples=3, desc_dist_threshold=2, color_dist_threshold=40,
             rel_lbsp_threshold=0.5)


# ---- ViBe (BackgroundSubtractorViBe.cpp: _1ch / _3ch) ----
@pytest.mark.parametrize("config,channels", [(0, 3), (0, 1), (2, 1)])
def test_vibe(config, channels):
    kw = {"channels": channels} if config == 0 else {}
    fr = _frames(config, 12, 2, **kw)
    params = {} if config == 0 else {"color_dist_threshold": 12, "bg_samples": 25, "required_bg_samples": 3}
    port = pyoracle.OracleViBe(seed=31, impl="port", **params)
    ref = pyoracle.OracleViBe(seed=31, impl="reference", **params)
    port.initialize(fr[0])
    ref.initialize(fr[0])
    assert np.array_equal(port.samples(), ref.samples()), "after initialize"
    for t, f in enumerate(fr[1:], start=1):
        lr = [16.0, 1.0, 2.0, float(3 + t)][t % 4]
        mp, mr = port.apply(f, lr), ref.apply(f, lr)
        assert np.array_equal(mp, mr), "frame %d: mask differs at %d px" % (t, int((mp != mr).sum()))
        assert np.array_equal(port.samples(), ref.samples()), "frame %d: samples differ" % t
    assert np.array_equal(port.background(), ref.background())


# ---- PBAS (BackgroundSubtractorPBAS.cpp: _1ch / _3ch) ----
@pytest.mark.parametrize("config,channels", [(0, 3), (0, 1), (2, 1)])
def test_pbas(config, channels):
    kw = {"channels": channels} if config == 0 else {}
    fr = _frames(config, 12, 3, **kw)
    params = {} if config == 0 else {"color_dist_threshold": 20, "update_rate": 8.0, "bg_samples": 25,
                                     "required_bg_samples": 3}
    port = pyoracle.OraclePBAS(seed=37, impl="port", **params)
    ref = pyoracle.OraclePBAS(seed=37, impl="reference", **params)
    port.initialize(fr[0])
    ref.initialize(fr[0])
    names = ("SAMPLE_COLOR", "SAMPLE_GRAD", "R", "T", "D")
    for n in names:
        assert np.array_equal(port.state_map(n), ref.state_map(n)), "after initialize: %s" % n
    for t, f in enumerate(fr[1:], start=1):
        lr = [-1.0, 1.0, -1.0, 3.5][t % 4]  # <= 0: T(x); > 0: the override
        mp, mr = port.apply(f, lr), ref.apply(f, lr)
        assert np.array_equal(mp, mr), "frame %d: mask differs at %d px" % (t, int((mp != mr).sum()))
        for n in names:
            assert np.array_equal(port.state_map(n), ref.state_map(n)), "frame %d: %s differs" % (t, n)
        assert port.mean_grad() == ref.mean_grad(), "frame %d: mean gradient distance" % t
    assert np.array_equal(port.background(), ref.background())
    # initialize() again: new samples and maps, the former mean gradient distance kept
    port.initialize(fr[5])
    ref.initialize(fr[5])
    assert port.mean_grad() == ref.mean_grad() != 20.0
    for t, f in enumerate(fr[6:9], start=1):
        mp, mr = port.apply(f, -1.0), ref.apply(f, -1.0)
        assert np.array_equal(mp, mr), "again, frame %d: mask differs" % t
        for n in names:
            assert np.array_equal(port.state_map(n), ref.state_map(n)), "again, frame %d: %s differs" % (t, n)
