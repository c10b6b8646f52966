"""GPU parity tests of PBAS (BackgroundSubtractorPBAS_1ch / _3ch): the CUDA path through the C-ABI against
the oracle (oracle/pbas.c, itself pinned bit for bit to the reference's own PBAS by
tests/test_oracle_reference.py). Every frame compares the mask, the colour and gradient samples, the R, T
and D maps, the gradient image and the frame-level mean gradient distance. Learning-rate overrides of 1
make most background pixels write a neighbour's sample (self diffusion), so those frames need repair
rounds; frames without an override use the per-pixel update rates T(x)."""
import ctypes as C

import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorPBAS, LvException, SyntheticStream
from litiv_gb300 import _lib as L
from oracle import pyoracle

pytestmark = pytest.mark.gpu

NAMES = {"nInitColorDistThreshold": "color_dist_threshold", "fInitUpdateRate": "update_rate",
         "nBGSamples": "bg_samples", "nRequiredBGSamples": "required_bg_samples"}
# GPU map name -> oracle map name
MAPS = [("SAMPLE_COLOR", "SAMPLE_COLOR"), ("SAMPLE_GRAD", "SAMPLE_GRAD"), ("R", "R"), ("T", "T"),
        ("DMIN_LT", "D"), ("GRAD", "GRAD")]


def frames_of(config, n, seed, **kw):
    s = SyntheticStream(config, 0, seed, **kw)
    return [s.render(t) for t in range(n)]


def check_state(gpu, ora, what):
    for gname, oname in MAPS:
        g, o = gpu.state_map(gname), ora.state_map(oname)
        if not np.array_equal(g.ravel(), o.ravel()):
            raise AssertionError("%s: %s differs at %d values" % (what, gname, int((g.ravel() != o.ravel()).sum())))
    mg = float(gpu.state_map("MEAN_GRAD")[0])
    assert mg == ora.mean_grad(), "%s: mean gradient distance %r vs %r" % (what, mg, ora.mean_grad())


def run_pair(frames, seed, lrs, gpu=None, ora=None, **params):
    if gpu is None:
        gpu = BackgroundSubtractorPBAS(seed=seed, **params)
        ora = pyoracle.OraclePBAS(seed=seed, **{NAMES[k]: v for k, v in params.items()})
    gpu.initialize(frames[0])
    ora.initialize(frames[0])
    check_state(gpu, ora, "after initialize")
    for t, f in enumerate(frames[1:], start=1):
        mg, mo = gpu.apply(f, learningRateOverride=lrs[t]), ora.apply(f, lrs[t])
        if not np.array_equal(mg, mo):
            raise AssertionError("frame %d: mask differs at %d px" % (t, int((mg != mo).sum())))
        check_state(gpu, ora, "frame %d" % t)
    return gpu, ora


@pytest.mark.parametrize("channels", [1, 3])
def test_pbas_bitexact(channels):
    fr = frames_of(0, 20, 1, channels=channels)
    lrs = [[-1.0, 1.0, -1.0, 2.0, 0.0, 3.5, float("inf")][t % 7] for t in range(20)]
    gpu, ora = run_pair(fr, 51, lrs)
    assert np.array_equal(gpu.getBackgroundImage(), ora.background())
    assert gpu.scalars()["frame_idx"] == 19
    # initialize() again: new samples and maps, the former mean gradient distance kept
    run_pair(fr[10:16], 51, [-1.0, 1.0, -1.0, 1.0, -1.0, -1.0], gpu=gpu, ora=ora)


def test_pbas_gray_scene_parameters():
    s = SyntheticStream(2, 0, 3)
    fr = [s.render(t) for t in range(10)]
    run_pair(fr, 52, [1.0, -1.0] * 5, nInitColorDistThreshold=20, fInitUpdateRate=8.0, nBGSamples=25,
             nRequiredBGSamples=3)


def test_pbas_1080p():
    # the three-channel mean gradient distance is a float sum over the whole frame in raster order
    s = SyntheticStream(1, 0, 5)
    fr = [s.render(t) for t in range(4)]
    run_pair(fr, 53, [-1.0, 1.0, -1.0, 1.0])


def test_pbas_argument_checks():
    fr = frames_of(0, 3, 6)
    m = BackgroundSubtractorPBAS(seed=1)
    with pytest.raises(LvException) as ei:
        m.apply(fr[1])
    assert ei.value.status == L.NOT_INITIALIZED
    roi = np.full(fr[0].shape[:2], 255, np.uint8)
    st = L.lib().lvbgs_initialize(m.handle, C.c_void_p(fr[0].ctypes.data), fr[0].shape[1], fr[0].shape[0], 3, 0,
                                  C.c_void_p(roi.ctypes.data))
    assert st == L.UNSUPPORTED
    m.initialize(fr[0])
    assert m.getDefaultLearningRate() == -1.0
    assert L.lib().lvbgs_refresh_model(m.handle, 0.5, 0) == L.UNSUPPORTED
    out = np.empty(fr[0].shape, np.uint16)
    assert L.lib().lvbgs_get_background_descriptors(m.handle, out.ctypes.data_as(C.c_void_p)) == L.UNSUPPORTED
    ora = pyoracle.OraclePBAS(seed=1)
    ora.initialize(fr[0])
    assert np.array_equal(m.apply(fr[1]), ora.apply(fr[1]))
    assert np.array_equal(m.apply(fr[2]), ora.apply(fr[2]))
