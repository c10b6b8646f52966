"""Change-detection evaluation (modules/datasets: lv::BinClassif, lv::BinClassifMetrics).

CPU: the oracle's restatement against hand-computed counters and metrics, and the C-ABI metrics
(host code) against the oracle. GPU: the device counters against the oracle on masks and CDnet-coded
ground truth holding every special value (out of scope, unknown, shadow) with and without a ROI, from
host and from device memory, and the F-measure of a SuBSENSE run on the synthetic scene.
"""
import ctypes as C

import numpy as np
import pytest

from litiv_gb300 import _lib as L
from oracle import metrics as om


def test_oracle_counters_and_metrics_by_hand():
    mask = np.array([[255, 255, 0, 0, 255, 0, 255, 0]], np.uint8)
    gt = np.array([[255, 0, 255, 0, 85, 170, 50, 50]], np.uint8)
    c = om.accumulate(mask, gt)
    # TP: px0; FP: px1, px6 (shadow counts as negative); FN: px2; TN: px3, px7; DC: px4, px5; SE: px6
    assert c == [1, 2, 2, 1, 1, 2]
    roi = np.array([[255, 0, 255, 255, 255, 255, 255, 255]], np.uint8)
    assert om.accumulate(mask, gt, roi) == [1, 2, 1, 1, 1, 3]
    m = om.metrics([1, 2, 2, 1, 1, 2])
    assert m[0] == 0.5 and m[5] == pytest.approx(1 / 3) and m[4] == pytest.approx(50.0)
    assert m[6] == pytest.approx(2 * 0.5 * (1 / 3) / (0.5 + 1 / 3))
    assert om.metrics([0, 5, 0, 0, 0, 0])[7] == 0.0  # an empty marginal
    assert om.accumulate(mask, None) == [0, 0, 0, 0, 0, 8]


def test_capi_metrics_equal_the_oracle(product_lib):
    rng = np.random.default_rng(4)
    for _ in range(50):
        c = [int(v) for v in rng.integers(0, 10 ** rng.integers(1, 9), 6)]
        if rng.random() < 0.2:
            c[int(rng.integers(0, 4))] = 0
        out = (C.c_double * 8)()
        assert product_lib.lvbgs_classif_metrics((C.c_uint64 * 6)(*c), out) == L.OK
        assert list(out) == om.metrics(c)  # same operation order: identical doubles


def _coded_gt(rng, shape):
    gt = rng.choice(np.array([0, 255, 85, 170, 50], np.uint8), size=shape, p=[0.55, 0.25, 0.08, 0.07, 0.05])
    mask = np.where(rng.random(shape) < 0.35, 255, 0).astype(np.uint8)
    mask[rng.random(shape) < 0.02] = 7  # a non-binary value counts as negative
    return mask, gt


@pytest.mark.gpu
@pytest.mark.parametrize("with_roi", [False, True])
def test_device_counters_equal_the_oracle(with_roi):
    from litiv_gb300.metrics import BinClassif
    rng = np.random.default_rng(9)
    for shape in [(37, 53), (480, 640), (1080, 1920)]:
        mask, gt = _coded_gt(rng, shape)
        roi = np.where(rng.random(shape) < 0.8, 255, 0).astype(np.uint8) if with_roi else None
        want = om.accumulate(mask, gt, roi)
        got = BinClassif().accumulate(mask, gt, roi)
        assert [int(v) for v in got.counts] == want
        assert list(got.metrics().values()) == om.metrics(want)


@pytest.mark.gpu
def test_device_counters_from_device_memory_accumulate():
    torch = pytest.importorskip("torch")
    from litiv_gb300.metrics import BinClassif
    rng = np.random.default_rng(10)
    mask, gt = _coded_gt(rng, (240, 320))
    bc = BinClassif()
    bc.accumulate(torch.from_numpy(mask).cuda(), torch.from_numpy(gt).cuda())
    bc.accumulate(mask, gt)
    want = om.accumulate(mask, gt, counts=om.accumulate(mask, gt))
    assert [int(v) for v in bc.counts] == want


@pytest.mark.gpu
def test_subsense_run_scored_on_the_device():
    from litiv_gb300 import BackgroundSubtractorSuBSENSE, SyntheticStream
    from litiv_gb300.metrics import BinClassif
    s = SyntheticStream(0, seed=2)
    b = BackgroundSubtractorSuBSENSE(seed=11)
    b.initialize(s.render(0))
    bc, want = BinClassif(), [0] * 6
    for t in range(1, 41):
        f, g = s.render(t, with_gt=True)
        m = b.apply(f)
        if t > 15:
            bc.accumulate(m, g)
            want = om.accumulate(m, g, counts=want)
    assert [int(v) for v in bc.counts] == want
    assert bc.metrics()["dFMeasure"] > 0.4
