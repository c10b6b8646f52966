"""GPU parity tests: the CUDA path (through the C-ABI) against the oracle, bit-exact.

Integer state, masks and descriptors must be identical; the FP32 feedback maps must be identical
too (tolerance 0 ulp), since both sides use the reference's operation order without fused
multiply-adds. Every frame compares every model map; the first mismatch is reported.
"""
import os

import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorSuBSENSE, LvException, SyntheticStream, batch_apply, lbsp_compute2
from oracle import pyoracle
from tests.helpers import compare_state

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MAX_ULP = 0  # FP32 tolerance of the feedback maps


def run_pair(frames, seed=5, lrs=None, roi=None, check_every=1, with_samples=True, **params):
    gpu = BackgroundSubtractorSuBSENSE(seed=seed, **params)
    ora = pyoracle.OracleSuBSENSE(seed=seed, **{_oname(k): v for k, v in params.items()})
    gpu.initialize(frames[0], roi)
    ora.initialize(frames[0], roi)
    bad = compare_state(gpu, ora, with_samples=with_samples)
    assert not bad, "after initialize: " + "; ".join(bad)
    for t, f in enumerate(frames[1:], start=1):
        lr = 0.0 if lrs is None else lrs[t]
        mg = gpu.apply(f, learningRateOverride=lr)
        mo = ora.apply(f, lr)
        assert np.array_equal(mg, mo), "frame %d: mask differs at %d px" % (t, int((mg != mo).sum()))
        if t % check_every == 0 or t == len(frames) - 1:
            bad = compare_state(gpu, ora, with_samples=with_samples)
            assert not bad, "frame %d: %s" % (t, "; ".join(bad))
    return gpu, ora


def _oname(k):
    return {"nDescDistThresholdOffset": "desc_dist_threshold_offset",
            "nMinColorDistThreshold": "min_color_dist_threshold", "nBGSamples": "bg_samples",
            "nRequiredBGSamples": "required_bg_samples", "nSamplesForMovingAvgs": "samples_for_moving_avgs",
            "fRelLBSPThreshold": "rel_lbsp_threshold",
            "nDefaultMedianBlurKernelSize": "default_median_blur_kernel_size"}[k]


def frames_of(stream, n, t0=0):
    return [stream.render(t) for t in range(t0, t0 + n)]


def test_lbsp_golden_vector_on_gpu():
    img = np.load(os.path.join(GOLDEN, "lbsp_input_65x65_bgr.npy"))
    gold = np.load(os.path.join(GOLDEN, "lbsp_abs20_65x65_u16c3.npy"))
    desc = lbsp_compute2(img, abs_threshold=20)
    np.testing.assert_array_equal(desc[2:-2, 2:-2], gold[2:-2, 2:-2])


@pytest.mark.parametrize("channels", [1, 3])
def test_lbsp_relative_matches_oracle(channels):
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (53, 67, channels) if channels == 3 else (53, 67), dtype=np.uint8)
    g = lbsp_compute2(img, rel_threshold=0.333, offset=2)
    o = pyoracle.lbsp_compute2(img, rel_threshold=0.333, offset=2)
    np.testing.assert_array_equal(g[2:-2, 2:-2], o[2:-2, 2:-2])


def test_subsense_small_frame_bitexact():
    """Small frame (frame-level analysis off, T caps x2, 9x9 median): every map, every frame."""
    s = SyntheticStream(0, seed=3, width=48, height=40, shape_min=6, shape_max=14)
    run_pair(frames_of(s, 25), seed=9)


def test_subsense_config0_bitexact():
    """320x240 BGR (config 0 shape): masks and all model state bit-exact over 60 frames."""
    s = SyntheticStream(0, seed=1)
    run_pair(frames_of(s, 61), seed=1, check_every=5)


def test_subsense_gray_bitexact():
    s = SyntheticStream(0, seed=8, channels=1)
    run_pair(frames_of(s, 31), seed=2, check_every=5)


def test_subsense_learning_rate_override_bitexact():
    """lr=1 for the first frames (the changedet app's schedule, apps/changedet/src/main.cpp:390):
    every background pixel updates itself and a neighbour, the densest raster-order dependencies."""
    s = SyntheticStream(0, seed=4, width=96, height=72, shape_min=10, shape_max=24)
    frames = frames_of(s, 31)
    lrs = [1.0 if t <= 20 else 0.0 for t in range(len(frames))]
    run_pair(frames, seed=4, lrs=lrs)


def test_subsense_roi_bitexact():
    s = SyntheticStream(0, seed=6)
    roi = np.zeros((240, 320), np.uint8)
    roi[30:210, 50:270] = 255
    roi[100:140, 120:200] = 0
    run_pair(frames_of(s, 21), seed=6, roi=roi, check_every=4)


def test_subsense_auto_model_reset_bitexact():
    """A sudden global intensity jump triggers the frame-level reset: refreshModel(0.1), T := 1."""
    s = SyntheticStream(0, seed=12)
    frames = frames_of(s, 48)
    # +150 from frame 30 (before frame 25 the long- and short-term averages share one factor, so a
    # change there cannot separate them); the reset fires at frame 43
    for t in range(30, 48):
        frames[t] = np.clip(frames[t].astype(np.int16) + 150, 0, 255).astype(np.uint8)
    gpu, ora = run_pair(frames, seed=12, check_every=1)
    assert ora.scalars()["model_reset_cooldown"] > 0  # the reset happened
    assert gpu.scalars()["lr_lower_cap"] == 1.0


def test_batched_streams_match_individual_runs():
    """Three streams of different sizes / channel counts batched into one set of phase kernels per tick."""
    streams = [SyntheticStream(0, seed=21), SyntheticStream(0, seed=22, channels=1, width=160, height=120),
               SyntheticStream(0, seed=23, width=64, height=48, shape_min=8, shape_max=16)]
    frames = [frames_of(s, 16) for s in streams]
    gpus = [BackgroundSubtractorSuBSENSE(seed=100 + i) for i in range(3)]
    oras = [pyoracle.OracleSuBSENSE(seed=100 + i) for i in range(3)]
    for g, o, f in zip(gpus, oras, frames):
        g.initialize(f[0])
        o.initialize(f[0])
    for t in range(1, 16):
        masks = batch_apply(gpus, [f[t] for f in frames])
        for i in range(3):
            mo = oras[i].apply(frames[i][t])
            assert np.array_equal(masks[i], mo), "stream %d frame %d" % (i, t)
    for g, o in zip(gpus, oras):
        assert not compare_state(g, o)


def test_background_images_and_manual_refresh():
    s = SyntheticStream(0, seed=31)
    frames = frames_of(s, 12)
    gpu, ora = run_pair(frames, seed=31, check_every=100)
    np.testing.assert_array_equal(gpu.getBackgroundImage(), ora.background())
    np.testing.assert_array_equal(gpu.getBackgroundDescriptorsImage(), ora.background_descriptors())
    gpu.refreshModel(0.3)
    ora.refresh_model(0.3)
    gpu.refreshModel(1.0, True)
    ora.refresh_model(1.0, True)
    assert not compare_state(gpu, ora)
    f = s.render(12)
    assert np.array_equal(gpu.apply(f), ora.apply(f))
    assert not compare_state(gpu, ora)


def test_spill_restore_is_transparent():
    s = SyntheticStream(0, seed=41, width=128, height=96)
    frames = frames_of(s, 14)
    a = BackgroundSubtractorSuBSENSE(seed=3)
    b = BackgroundSubtractorSuBSENSE(seed=3)
    a.initialize(frames[0])
    b.initialize(frames[0])
    for t in range(1, 14):
        if t == 7:
            buf = bytearray(a.state_bytes())
            a.spill(buf)
            with pytest.raises(LvException):
                a.apply(frames[t])
            a.restore(buf)
        assert np.array_equal(a.apply(frames[t]), b.apply(frames[t]))


def test_api_errors():
    g = BackgroundSubtractorSuBSENSE()
    with pytest.raises(LvException):
        g.apply(np.zeros((20, 20, 3), np.uint8))
    with pytest.raises(LvException):
        g.initialize(np.zeros((20, 20, 3), np.uint8), np.full((20, 20), 3, np.uint8))
    g.initialize(np.zeros((20, 20, 3), np.uint8))
    with pytest.raises(LvException):
        g.apply(np.zeros((21, 20, 3), np.uint8))
    with pytest.raises(LvException):
        g.refreshModel(0.0)
    assert g.getDefaultLearningRate() == 0.0


@pytest.mark.parametrize("channels", [1, 3])
def test_odd_width_wide_median(channels):
    # 70 px rows: the bit planes end in a partial word (6 bits) and the rows of the byte maps are not
    # 4-byte aligned; a 15x15 median (row window 15, sliding column sums over 15 rows)
    s = SyntheticStream(0, seed=51, width=70, height=50, shape_min=8, shape_max=20, channels=channels)
    run_pair(frames_of(s, 24), seed=52, nDefaultMedianBlurKernelSize=15)


def test_frame_level_analysis_with_partial_words():
    # 344x256: large enough for the frame-level analysis (integral 1/8 down-sampling: 43x32 blocks of
    # 8x8) while the rows end in a partial 24-bit word; median 9
    s = SyntheticStream(0, seed=53, width=344, height=256)
    run_pair(frames_of(s, 14), seed=54, check_every=6)



def _ellipse_roi(W, H):
    yy, xx = np.mgrid[0:H, 0:W]
    return ((((xx - W / 2) / (W * 0.42)) ** 2 + ((yy - H / 2) / (H * 0.42)) ** 2) <= 1.0).astype(np.uint8) * 255


def _step_and_compare(gpu, ora, frames, t0):
    for t, f in enumerate(frames, start=t0):
        mg, mo = gpu.apply(f), ora.apply(f, 0.0)
        assert np.array_equal(mg, mo), "frame %d: mask differs at %d px" % (t, int((mg != mo).sum()))
    bad = compare_state(gpu, ora)
    assert not bad, "; ".join(bad)


def test_set_roi_reinitializes_from_background():
    # setROI on an initialized model: initialize(getBackgroundImage(), validated ROI)
    s = SyntheticStream(0, seed=61, width=96, height=72, shape_min=10, shape_max=24)
    fr = frames_of(s, 16)
    gpu, ora = BackgroundSubtractorSuBSENSE(seed=62), pyoracle.OracleSuBSENSE(seed=62)
    gpu.initialize(fr[0])
    ora.initialize(fr[0])
    _step_and_compare(gpu, ora, fr[1:6], 1)
    roi = _ellipse_roi(96, 72)
    gpu.setROI(roi)
    ora.set_roi(roi)
    assert np.array_equal(gpu.getROICopy(), ora.state_map("ROI"))
    assert not compare_state(gpu, ora)
    _step_and_compare(gpu, ora, fr[6:], 6)


def test_set_roi_before_initialize_and_roi_reuse():
    # a ROI set before initialize() is used as is (validated, not dilated); a later initialize()
    # without a ROI of the same size reuses the last validated ROI
    s = SyntheticStream(0, seed=63, width=96, height=72, shape_min=10, shape_max=24)
    fr = frames_of(s, 14)
    gpu, ora = BackgroundSubtractorSuBSENSE(seed=64), pyoracle.OracleSuBSENSE(seed=64)
    roi = _ellipse_roi(96, 72)
    gpu.setROI(roi)
    ora.set_roi(roi)
    gpu.initialize(fr[0])
    ora.initialize(fr[0])
    assert np.array_equal(gpu.getROICopy(), gpu.validateROI(roi))
    assert not compare_state(gpu, ora)
    _step_and_compare(gpu, ora, fr[1:7], 1)
    gpu.initialize(fr[7])
    ora.initialize(fr[7])
    assert np.array_equal(gpu.getROICopy(), gpu.validateROI(roi))
    assert not compare_state(gpu, ora)
    _step_and_compare(gpu, ora, fr[8:], 8)
    assert gpu.isParallel() and gpu.getParallelAlgoType() == "CUDA"
    with pytest.raises(LvException):
        gpu.setROI(np.zeros((72, 96), np.uint8))


@pytest.mark.parametrize("groups", [2, 4])
def test_split_batch_groups_equal_streams_alone(groups):
    # >= 8 streams and >= 4 Mi pixels: lvbgs_batch_apply runs the batch as concurrent groups (one CUDA
    # stream each, repair grids of 1/groups of the device); every mask and model map must equal the
    # stream alone
    from litiv_gb300 import _lib
    lib = _lib.lib()
    assert lib.lvbgs_set_batch_groups(groups) == 0
    try:
        _split_batch_case(groups)
    finally:
        lib.lvbgs_set_batch_groups(4)


def _split_batch_case(groups):
    specs = [(1280, 720, 3)] * 4 + [(640, 480, 1)] * (8 if groups > 2 else 4) + [(320, 240, 3)] * (4 if groups > 2 else 2)
    streams = [SyntheticStream(0, seed=71 + i, width=W, height=H, channels=Cn) for i, (W, H, Cn) in enumerate(specs)]
    frames = [frames_of(s, 6) for s in streams]
    batched = [BackgroundSubtractorSuBSENSE(seed=200 + i) for i in range(len(specs))]
    alone = [BackgroundSubtractorSuBSENSE(seed=200 + i) for i in range(len(specs))]
    for b, a, f in zip(batched, alone, frames):
        b.initialize(f[0])
        a.initialize(f[0])
    for t in range(1, 6):
        masks = batch_apply(batched, [f[t] for f in frames])
        for i in range(len(specs)):
            assert np.array_equal(masks[i], alone[i].apply(frames[i][t])), "stream %d frame %d" % (i, t)
    for b, a in zip(batched, alone):
        for name in ("R", "T", "V", "DMIN_LT", "UNSTABLE", "LAST_FG", "SAMPLE_COLOR", "SAMPLE_DESC"):
            assert np.array_equal(b.state_map(name), a.state_map(name)), name


@pytest.mark.parametrize("W,H", [(640, 350), (595, 245)])
def test_non_integral_down_sampling_bitexact(W, H):
    """Frame sizes whose 1/8 frame-level down-sampling is not integral (INTER_AREA as the exact
    area-weighted mean, :568): masks and every map, including the down-sampled means."""
    s = SyntheticStream(0, seed=42, width=W, height=H)
    run_pair(frames_of(s, 16), seed=14, check_every=3)


def test_page_locked_host_masks_are_written_by_the_kernels():
    """Masks into page-locked host memory (written by the post-processing kernel itself over the host
    link, no copy after the step) equal the masks written into pageable memory (device staging buffer
    and a copy), for a batch of streams, a single SuBSENSE stream and a PAWCS stream."""
    torch = pytest.importorskip("torch")
    from litiv_gb300 import BackgroundSubtractorPAWCS
    streams = [SyntheticStream(0, seed=61), SyntheticStream(0, seed=62, channels=1, width=160, height=120)]
    frames = [frames_of(s, 8) for s in streams]
    runs = []
    for pinned in (False, True):
        subs = [BackgroundSubtractorSuBSENSE(seed=70 + i) for i in range(2)]
        single = BackgroundSubtractorSuBSENSE(seed=80)
        pw = BackgroundSubtractorPAWCS(seed=81)
        for g, f in zip(subs, frames):
            g.initialize(f[0])
        single.initialize(frames[0][0])
        pw.initialize(frames[1][0])

        def buf(shape):
            if pinned:
                return torch.empty(shape, dtype=torch.uint8).pin_memory().numpy()
            return np.empty(shape, np.uint8)

        out = []
        for t in range(1, 8):
            masks = batch_apply(subs, [f[t] for f in frames], masks=[buf(f[t].shape[:2]) for f in frames])
            m1 = single.apply(frames[0][t], fgmask=buf(frames[0][t].shape[:2]))
            m2 = pw.apply(frames[1][t], fgmask=buf(frames[1][t].shape[:2]))
            out.append([m.copy() for m in masks] + [m1.copy(), m2.copy()])
        runs.append(out)
    for t, (a, b) in enumerate(zip(*runs), start=1):
        for i, (ma, mb) in enumerate(zip(a, b)):
            assert np.array_equal(ma, mb), "frame %d, output %d differs between pageable and page-locked masks" % (t, i)
    assert any(m.any() for o in runs[1] for m in o), "no foreground at all: the comparison says nothing"
