"""GPU parity tests of LOBSTER (one and three channels): the CUDA path through the C-ABI against the
oracle (oracle/lobster.c, itself pinned bit for bit to the reference's own
BackgroundSubtractorLOBSTER by tests/test_oracle_reference.py).

Masks must be identical on every frame, and the whole model (every sample colour and descriptor, the
last colour and descriptor frames, the last mask) on the checked frames. The learning rate 1 cases
make every background pixel write a neighbour's sample, so most frames need the raster-order repair.
"""
import ctypes as C

import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorLOBSTER, LvException, SyntheticStream
from litiv_gb300 import _lib as L
from oracle import pyoracle

pytestmark = pytest.mark.gpu

MAPS = ["LAST_FG", "ROI", "LAST_COLOR", "LAST_DESC", "SAMPLE_COLOR", "SAMPLE_DESC", "LUT"]

_PARAM_NAMES = {"nDescDistThreshold": "desc_dist_threshold", "nColorDistThreshold": "color_dist_threshold",
                "nBGSamples": "bg_samples", "nRequiredBGSamples": "required_bg_samples",
                "fRelLBSPThreshold": "rel_lbsp_threshold", "nLBSPThresholdOffset": "lbsp_threshold_offset"}


def compare_state(gpu, ora, where):
    for name in MAPS:
        a = np.asarray(gpu.state_map(name)).view(np.uint8).ravel()
        b = np.asarray(ora.state_map(name)).view(np.uint8).ravel()
        assert a.size == b.size, "%s: %s sizes differ" % (where, name)
        if not np.array_equal(a, b):
            idx = np.flatnonzero(a != b)
            raise AssertionError("%s: %s differs in %d bytes (first at byte %d)" % (where, name, idx.size, idx[0]))
    sg, so = gpu.scalars(), ora.scalars()
    assert sg["frame_idx"] == so["frames"] and sg["n_relevant_px"] == so["n_relevant_px"], where
    assert sg["stat_sample_writes"] == so["stat_sample_writes"], where


def run_pair(frames, seed=5, lrs=None, roi=None, check_every=1, refreshes=(), **params):
    gpu = BackgroundSubtractorLOBSTER(seed=seed, **params)
    ora = pyoracle.OracleLOBSTER(seed=seed, **{_PARAM_NAMES[k]: v for k, v in params.items()})
    gpu.initialize(frames[0], roi)
    ora.initialize(frames[0], roi)
    compare_state(gpu, ora, "after initialize")
    for t, f in enumerate(frames[1:], start=1):
        lr = 16.0 if lrs is None else lrs[t]
        mg, mo = gpu.apply(f, learningRate=lr), ora.apply(f, lr)
        if not np.array_equal(mg, mo):
            raise AssertionError("frame %d: mask differs at %d px" % (t, int((mg != mo).sum())))
        if t % check_every == 0 or t == len(frames) - 1:
            compare_state(gpu, ora, "frame %d" % t)
        for (ti, frac, force) in refreshes:
            if ti == t:
                gpu.refreshModel(frac, force)
                ora.refresh_model(frac, force)
                compare_state(gpu, ora, "refresh after frame %d" % t)
    return gpu, ora


def frames_of(config, n, seed, **kw):
    s = SyntheticStream(config, 0, seed, **kw)
    return [s.render(t) for t in range(n)]


def test_lobster_bgr_scene_bitexact():
    # the 320x240 BGR scene of moving shapes, the reference's default learning rate
    run_pair(frames_of(0, 40, 1), seed=11, check_every=5)


def test_lobster_gray_scene_bitexact():
    run_pair(frames_of(2, 16, 2), seed=12, check_every=5)


@pytest.mark.parametrize("channels", [1, 3])
def test_lobster_fast_learning_needs_repair(channels):
    # learning rate 1: every background pixel updates its own and a neighbour's sample, so earlier
    # pixels overwrite the samples later ones read in almost every frame
    fr = frames_of(0, 14, 3, channels=channels)
    lrs = [1.0] * 14
    run_pair(fr, seed=13, lrs=lrs, check_every=1)


def test_lobster_learning_rates_roi_refresh_and_background_images():
    fr = frames_of(0, 16, 4)
    roi = np.zeros(fr[0].shape[:2], np.uint8)
    roi[20:200, 30:290] = 255
    lrs = [16.0, 1.0, 1.0, 2.0, 3.5, 16.0, float("inf"), 1.0, 4.0, 16.0, 1.0, 2.0, 16.0, 1.0, 5.0, 1.0]
    gpu, ora = run_pair(fr, seed=14, lrs=lrs, roi=roi, refreshes=((5, 0.4, False), (9, 1.0, True), (12, 0.1, False)))
    assert np.array_equal(gpu.getBackgroundImage(), ora.background())
    assert np.array_equal(gpu.getBackgroundDescriptorsImage(), ora.background_descriptors())


def test_lobster_parameters():
    fr = frames_of(0, 12, 5, channels=1)
    run_pair(fr, seed=15, lrs=[2.0] * 12, nBGSamples=20, nRequiredBGSamples=3, nDescDistThreshold=2,
             nColorDistThreshold=40, fRelLBSPThreshold=0.5)


def test_lobster_1080p_prefix():
    s = SyntheticStream(1, 0, 6)
    fr = [s.render(t) for t in range(6)]
    run_pair(fr, seed=16, lrs=[1.0, 1.0, 16.0, 1.0, 2.0, 1.0], check_every=5)


def test_lobster_argument_checks():
    fr = frames_of(0, 3, 7)
    m = BackgroundSubtractorLOBSTER(seed=1)
    with pytest.raises(LvException) as ei:
        m.apply(fr[1])
    assert ei.value.status == L.NOT_INITIALIZED
    m.initialize(fr[0])
    assert m.getDefaultLearningRate() == 16.0
    for bad in (0.0, -1.0, float("nan")):
        with pytest.raises(LvException) as ei:
            m.apply(fr[1], learningRate=bad)
        assert ei.value.status == L.BAD_ARG
    with pytest.raises(LvException) as ei:
        m.refreshModel(0.0)
    assert ei.value.status == L.BAD_ARG
    buf = np.empty(1 << 20, np.uint8)
    assert L.lib().lvbgs_spill(m.handle, buf.ctypes.data_as(C.c_void_p), buf.size) == L.UNSUPPORTED
    # the model still works after the refused calls
    ora = pyoracle.OracleLOBSTER(seed=1)
    ora.initialize(fr[0])
    assert np.array_equal(m.apply(fr[1]), ora.apply(fr[1]))
    assert np.array_equal(m.apply(fr[2]), ora.apply(fr[2]))
