"""GPU parity tests of ViBe (BackgroundSubtractorViBe_1ch / _3ch): the CUDA path through the C-ABI against
the oracle (oracle/vibe.c, itself pinned bit for bit to the reference's own ViBe by
tests/test_oracle_reference.py). Masks are compared on every frame and all samples on every frame; the
learning rate 1 frames make most background pixels write a neighbour's sample, so they need repair
rounds."""
import ctypes as C

import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorViBe, LvException, SyntheticStream
from litiv_gb300 import _lib as L
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def frames_of(config, n, seed, **kw):
    s = SyntheticStream(config, 0, seed, **kw)
    return [s.render(t) for t in range(n)]


def run_pair(frames, seed, lrs, **params):
    names = {"nColorDistThreshold": "color_dist_threshold", "nBGSamples": "bg_samples",
             "nRequiredBGSamples": "required_bg_samples"}
    gpu = BackgroundSubtractorViBe(seed=seed, **params)
    ora = pyoracle.OracleViBe(seed=seed, **{names[k]: v for k, v in params.items()})
    gpu.initialize(frames[0])
    ora.initialize(frames[0])
    assert np.array_equal(gpu.state_map("SAMPLE_COLOR").ravel(), ora.samples().ravel()), "after initialize"
    for t, f in enumerate(frames[1:], start=1):
        mg, mo = gpu.apply(f, learningRate=lrs[t]), ora.apply(f, lrs[t])
        if not np.array_equal(mg, mo):
            raise AssertionError("frame %d: mask differs at %d px" % (t, int((mg != mo).sum())))
        if not np.array_equal(gpu.state_map("SAMPLE_COLOR").ravel(), ora.samples().ravel()):
            raise AssertionError("frame %d: samples differ" % t)
    stats = ora.stats()
    sc = gpu.scalars()
    assert sc["frame_idx"] == stats[0] and sc["stat_sample_writes"] == stats[2]
    return gpu, ora


@pytest.mark.parametrize("channels", [1, 3])
def test_vibe_bitexact(channels):
    fr = frames_of(0, 24, 1, channels=channels)
    lrs = [[16.0, 1.0, 2.0, 16.0, float("inf"), 4.5][t % 6] for t in range(24)]
    gpu, ora = run_pair(fr, 41, lrs)
    assert np.array_equal(gpu.getBackgroundImage(), ora.background())


def test_vibe_gray_scene_parameters():
    s = SyntheticStream(2, 0, 3)
    fr = [s.render(t) for t in range(10)]
    run_pair(fr, 42, [1.0] * 10, nColorDistThreshold=12, nBGSamples=25, nRequiredBGSamples=3)


def test_vibe_wide_threshold_and_1080p():
    # 3R >= 256: every sample matches on three channels
    fr = frames_of(0, 5, 4)
    run_pair(fr, 43, [1.0] * 5, nColorDistThreshold=90)
    s = SyntheticStream(1, 0, 5)
    fr = [s.render(t) for t in range(4)]
    run_pair(fr, 44, [1.0, 1.0, 16.0, 1.0])


def test_vibe_argument_checks():
    fr = frames_of(0, 3, 6)
    m = BackgroundSubtractorViBe(seed=1)
    with pytest.raises(LvException) as ei:
        m.apply(fr[1])
    assert ei.value.status == L.NOT_INITIALIZED
    roi = np.full(fr[0].shape[:2], 255, np.uint8)
    st = L.lib().lvbgs_initialize(m.handle, C.c_void_p(fr[0].ctypes.data), fr[0].shape[1], fr[0].shape[0], 3, 0,
                                  C.c_void_p(roi.ctypes.data))
    assert st == L.UNSUPPORTED
    m.initialize(fr[0])
    assert m.getDefaultLearningRate() == 16.0
    with pytest.raises(LvException) as ei:
        m.apply(fr[1], learningRate=0.0)
    assert ei.value.status == L.BAD_ARG
    assert L.lib().lvbgs_refresh_model(m.handle, 0.5, 0) == L.UNSUPPORTED
    ora = pyoracle.OracleViBe(seed=1)
    ora.initialize(fr[0])
    assert np.array_equal(m.apply(fr[1]), ora.apply(fr[1]))
    assert np.array_equal(m.apply(fr[2]), ora.apply(fr[2]))
