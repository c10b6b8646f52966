"""Failure detection on the GPU, tested without a fault.

The device-side waits of a frame step are bounded: the cooperative repair kernel's grid barrier
gives up after a time limit (LVBGS_DEVICE_TIMEOUT), the raster-order repair after a round limit and
PAWCS's fixed point after a round limit (LVBGS_DEVICE_ERROR). lvbgs_debug_inject_fault makes one of
these limits run out in the next frame step of a handle (a barrier that one CTA never reaches, with a
2 ms limit; a round limit of zero or one), so each test checks that the kernels return, that the call
reports the status, and that the context and the other handles keep working: their next frames still
equal the oracle bit for bit, and the failed handle works again after initialize().
"""
import ctypes as C
import time

import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorPAWCS, BackgroundSubtractorSuBSENSE, LvException, SyntheticStream
from litiv_gb300 import _lib as L
from litiv_gb300 import batch_apply
from oracle import pyoracle

pytestmark = pytest.mark.gpu

FAULT_BARRIER_TIMEOUT, FAULT_REPAIR_LIMIT, FAULT_PAWCS_ROUNDS = 1, 2, 3


def _inject(model, kind):
    assert L.lib().lvbgs_debug_inject_fault(model.handle, kind) == L.OK


def _frames(n, seed, channels=3, **kw):
    s = SyntheticStream(0, 0, seed, width=96, height=72, shape_min=10, shape_max=24, channels=channels, **kw)
    return [s.render(t) for t in range(n)]


def _pair(cls, ocls, seed, frame0):
    g, o = cls(seed=seed), ocls(seed=seed)
    g.initialize(frame0)
    o.initialize(frame0)
    return g, o


def _same_next_frames(g, o, frames, lr=0.0):
    for t, f in enumerate(frames):
        mg, mo = g.apply(f, learningRateOverride=lr), o.apply(f, lr)
        assert np.array_equal(mg, mo), "frame %d after the injected failure differs from the oracle" % t


@pytest.mark.parametrize("kind,status", [(FAULT_BARRIER_TIMEOUT, L.DEVICE_TIMEOUT), (FAULT_REPAIR_LIMIT, L.DEVICE_ERROR)])
def test_subsense_wait_gives_up_and_reports(kind, status):
    fr = _frames(14, 51)
    # lr = 1: every background pixel writes itself and a neighbour, so frames need repair rounds; a
    # twin run without the fault finds the first frame that does
    twin = BackgroundSubtractorSuBSENSE(seed=5)
    twin.initialize(fr[0])
    k = None
    for t in range(1, 8):
        before = twin.scalars()["stat_repair_rematched"]
        twin.apply(fr[t], learningRateOverride=1.0)
        if twin.scalars()["stat_repair_rematched"] > before:
            k = t
            break
    assert k is not None, "no frame needs a repair round"

    victim = BackgroundSubtractorSuBSENSE(seed=5)
    victim.initialize(fr[0])
    other, ora = _pair(BackgroundSubtractorSuBSENSE, pyoracle.OracleSuBSENSE, 6, fr[0])
    for f in fr[1:k]:
        victim.apply(f, learningRateOverride=1.0)
    _same_next_frames(other, ora, fr[1:k], lr=1.0)
    _inject(victim, kind)
    t0 = time.perf_counter()
    with pytest.raises(LvException) as ei:
        victim.apply(fr[k], learningRateOverride=1.0)
    assert ei.value.status == status
    assert time.perf_counter() - t0 < 1.5  # the 2 ms limit, not the 2 s one
    # the context and the other handle keep working
    _same_next_frames(other, ora, fr[k:k + 5], lr=1.0)
    # the failed handle works again after initialize()
    victim.initialize(fr[k + 1])
    o2 = pyoracle.OracleSuBSENSE(seed=5)
    o2.initialize(fr[k + 1])
    _same_next_frames(victim, o2, fr[k + 2:k + 6])


def test_batched_step_reports_the_barrier_timeout():
    fr = [_frames(8, 60 + i) for i in range(3)]
    lead = [BackgroundSubtractorSuBSENSE(seed=20 + i) for i in range(3)]
    for m, f in zip(lead, fr):
        m.initialize(f[0])
    other, ora = _pair(BackgroundSubtractorSuBSENSE, pyoracle.OracleSuBSENSE, 30, fr[0][0])
    _inject(lead[0], FAULT_BARRIER_TIMEOUT)
    with pytest.raises(LvException) as ei:
        batch_apply(lead, [f[1] for f in fr])
    assert ei.value.status == L.DEVICE_TIMEOUT
    _same_next_frames(other, ora, fr[0][1:8])
    # the next batched step of re-initialized streams succeeds
    for m, f in zip(lead, fr):
        m.initialize(f[2])
    masks = batch_apply(lead, [f[3] for f in fr])
    for i, f in enumerate(fr):
        o = pyoracle.OracleSuBSENSE(seed=20 + i)
        o.initialize(f[2])
        assert np.array_equal(masks[i], o.apply(f[3]))


@pytest.mark.parametrize("channels", [1, 3])
def test_pawcs_fixed_point_round_limit_reports(channels):
    fr = _frames(12, 70, channels=channels)
    twin = BackgroundSubtractorPAWCS(seed=7)
    twin.initialize(fr[0])
    k = None
    for t in range(1, 8):
        twin.apply(fr[t])
        if twin.scalars()["fixed_point_rounds"] > 1:
            k = t
            break
    assert k is not None, "every frame converges in one round"
    victim = BackgroundSubtractorPAWCS(seed=7)
    victim.initialize(fr[0])
    other, ora = _pair(BackgroundSubtractorPAWCS, pyoracle.OraclePAWCS, 8, fr[0])
    for f in fr[1:k]:
        victim.apply(f)
    _inject(victim, FAULT_PAWCS_ROUNDS)
    with pytest.raises(LvException) as ei:
        victim.apply(fr[k])
    assert ei.value.status == L.DEVICE_ERROR
    _same_next_frames(other, ora, fr[1:12])


def test_inject_fault_argument_checks():
    lib = L.lib()
    assert lib.lvbgs_debug_inject_fault(None, FAULT_BARRIER_TIMEOUT) == L.BAD_ARG
    m = BackgroundSubtractorSuBSENSE(seed=1)
    assert lib.lvbgs_debug_inject_fault(m.handle, 99) == L.BAD_ARG
