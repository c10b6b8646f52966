"""GPU parity tests against the REFERENCE's own results on the full benchmark workloads.

tests/golden/parity_digests.json holds digests (BLAKE2b-128 of the raw bytes) of what the
reference's own SuBSENSE / PAWCS sources compute on the seeded synthetic scenes (generated by
tests/golden/make_parity_digests.py from oracle/_ref, the reference compiled against the
project-written OpenCV stand-in): the foreground mask of every frame and, at checkpoints, every model
map (samples, words, FP32 feedback maps at 0 ulp, ...) with the frame-level scalars. The CUDA path runs
the same frames through the C-ABI and must reproduce every digest:

  * config 0: 320x240 BGR, all 200 frames
  * config 1: 1920x1080 BGR, 300 of the 500 frames (13x13 median, 5x5 spread, ripple, drift, both
    stopped ellipses)
  * the changedet learning-rate schedule (lr = 1 for frames <= 100, apps/changedet/src/main.cpp:390)
    at 640x480 BGR
  * config 2: PAWCS on the 640x480 thermal-like scene, all 300 frames
  * config 3: the 64-stream mix through lvbgs_batch_apply (default four concurrent groups) over the
    benchmark's own streams and seeds, initialize + 30 ticks (the timed ticks of bench.py among them):
    every stream's mask of every tick, every stream's full state at the end
"""
import hashlib
import json
import os

import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorPAWCS, BackgroundSubtractorSuBSENSE, SyntheticStream, batch_apply

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "parity_digests.json")


def _doc():
    return json.load(open(GOLDEN))


def _digest(a):
    return hashlib.blake2b(np.ascontiguousarray(a).view(np.uint8).tobytes(), digest_size=16).hexdigest()


def _check_state(model, want, where):
    bad = [n for n, d in want["maps"].items() if _digest(model.state_map(n)) != d]
    sc = model.scalars()
    bad += ["scalar %s: %r vs %r" % (k, sc[k], v) for k, v in want["scalars"].items()
            if (float(sc[k]) if isinstance(v, float) else int(sc[k])) != v]
    assert not bad, "%s: differs from the reference in %s" % (where, bad)


def _run_case(name):
    case = _doc()["cases"][name]
    scene = SyntheticStream(case["config"], case["index"], case["scene_seed"], **case.get("scene", {}))
    cls = BackgroundSubtractorSuBSENSE if case["algo"] == "subsense" else BackgroundSubtractorPAWCS
    model = cls(seed=case["seed"])
    model.initialize(scene.render(0))
    _check_state(model, case["states"]["0"], "%s after initialize" % name)
    lrs = [1.0 if t <= 100 else 0.0 for t in range(case["n"])] if name == "subsense_changedet" else None
    for t in range(1, case["n"]):
        mask = model.apply(scene.render(t), learningRateOverride=0.0 if lrs is None else lrs[t])
        assert _digest(mask) == case["masks"][t - 1], "%s frame %d: mask differs from the reference" % (name, t)
        if str(t) in case["states"]:
            _check_state(model, case["states"][str(t)], "%s frame %d" % (name, t))
    model.close()


def test_subsense_config0_all_frames_match_the_reference():
    _run_case("subsense_config0")


def test_subsense_config1_1080p_matches_the_reference():
    _run_case("subsense_config1")


def test_subsense_changedet_schedule_matches_the_reference():
    _run_case("subsense_changedet")


def test_pawcs_config2_all_frames_match_the_reference():
    _run_case("pawcs_config2")


def test_subsense_mix64_batched_ticks_match_the_reference():
    case = _doc()["cases"]["subsense_mix64"]
    scenes = [SyntheticStream(3, i, case["scene_seed"]) for i in range(64)]
    models = [BackgroundSubtractorSuBSENSE(seed=case["seed_base"] + i) for i in range(64)]
    for m, s in zip(models, scenes):
        m.initialize(s.render(0))
    for t in range(1, case["ticks"] + 1):
        masks = batch_apply(models, [s.render(t) for s in scenes])
        bad = [i for i in range(64) if _digest(masks[i]) != case["streams"][i]["masks"][t - 1]]
        assert not bad, "tick %d: masks of streams %s differ from the reference" % (t, bad)
    for i, m in enumerate(models):
        _check_state(m, case["streams"][i]["states"][str(case["ticks"])], "mix64 stream %d" % i)
        m.close()
