"""Serving loop (include/lvserve.h): host policy on the CPU, continuous batching on the GPU.

The GPU tests check that each stream's masks are the same alone (lvbgs_apply, one stream) and in
the mix (served with other streams of other sizes and channel counts, under an HBM budget that
forces streams to wait for admission and idle streams to spill to host memory and come back).
Masks are integers: the tolerance is zero.
"""
import ctypes as C

import numpy as np
import pytest

from litiv_gb300 import _lib as L
from litiv_gb300 import serving
from litiv_gb300.synth import SyntheticStream

GiB = 1 << 30


def test_default_config_and_workload():
    cfg = serving.default_config()
    assert (cfg.max_live, cfg.max_queue, cfg.max_inflight, cfg.pawcs_lanes) == (256, 8, 2, 1)
    assert cfg.idle_spill_ms == 500.0
    sim = serving.default_sim_config()
    # Poisson arrivals at 4 streams/s, lives U[10, 60] s, 30 fps, resolution mix .3/.3/.3/.1
    assert (sim.arrival_rate, sim.life_min_s, sim.life_max_s, sim.fps) == (4.0, 10.0, 60.0, 30.0)
    assert [round(p, 6) for p in sim.res_prob] == [0.3, 0.3, 0.3, 0.1]
    # a quarter single-channel; 2.5 % of the streams (either channel count) run PAWCS (SuBSENSE/PAWCS mixed)
    assert (sim.gray_prob, sim.pawcs_prob) == (0.25, 0.025)


def test_create_rejects_bad_config():
    lib = L.lib()
    h = C.c_void_p()
    for field, value in [("max_live", 0), ("max_queue", 0), ("max_inflight", 0), ("max_inflight", 5),
                         ("idle_spill_ms", -1.0), ("pawcs_lanes", -1)]:
        cfg = serving.default_config(**{field: value})
        assert lib.lvserve_create(C.byref(cfg), C.byref(h)) == L.BAD_ARG, field
    assert lib.lvserve_submit(None, 1, None, 0, None, 0.0, 0) == L.BAD_ARG


def test_plan_room_fits_without_spilling():
    assert serving.plan_room(10 * GiB, 40 * GiB, 5 * GiB, [4 * GiB], [1e4], 500.0) == []


def test_plan_room_spills_longest_idle_first():
    # 35 GiB used of 40; 10 GiB needed: spill candidates by decreasing idle time until it fits
    bytes_ = [3 * GiB, 4 * GiB, 2 * GiB, 6 * GiB]
    idle = [900.0, 5000.0, 100.0, 2000.0]
    pick = serving.plan_room(35 * GiB, 40 * GiB, 10 * GiB, bytes_, idle, 500.0)
    assert pick == [1, 3]  # 4 + 6 GiB freed -> 25 + 10 <= 40
    # the stream idle for 100 ms is not eligible at a 500 ms threshold
    pick = serving.plan_room(35 * GiB, 40 * GiB, 16 * GiB, bytes_, idle, 500.0)
    assert pick == [1, 3, 0]
    assert serving.plan_room(35 * GiB, 40 * GiB, 19 * GiB, bytes_, idle, 500.0) is None


def test_plan_room_never_fits_an_oversized_need():
    assert serving.plan_room(0, 40 * GiB, 41 * GiB, [], [], 0.0) is None
    assert serving.plan_room(39 * GiB, 40 * GiB, 2 * GiB, [1 * GiB], [10.0], 0.0) == [0]


def test_device_bytes_cover_the_spill_image():
    lib = L.lib()
    for (W, H, Cn) in [(320, 240, 3), (640, 480, 1), (1920, 1080, 3)]:
        st = lib.lvbgs_state_bytes(L.ALGO_SUBSENSE, W, H, Cn, 50)
        dev = lib.lvbgs_device_bytes(L.ALGO_SUBSENSE, W, H, Cn, 50)
        assert 0 < st < dev
    assert lib.lvbgs_device_bytes(L.ALGO_SUBSENSE, 320, 240, 2, 50) == 0


# ------------------------------------------------------------------------------------------
# GPU
# ------------------------------------------------------------------------------------------
STREAMS = [  # (width, height, channels, seed)
    (64, 48, 3, 11),
    (96, 64, 1, 12),
    (160, 120, 3, 13),
    (128, 96, 3, 14),
]


def _frames(W, H, Cn, seed, n):
    s = SyntheticStream(0, 0, seed, width=W, height=H, channels=Cn)
    return [s.render(t) for t in range(n)]


def _alone(frames, seed):
    from litiv_gb300 import BackgroundSubtractorSuBSENSE
    b = BackgroundSubtractorSuBSENSE(seed=seed)
    b.initialize(frames[0])
    return [b.apply(f) for f in frames[1:]]


@pytest.mark.gpu
def test_served_masks_equal_alone_masks_with_waits_spills_and_restores():
    lib = L.lib()
    n_frames = 13
    data = [_frames(W, H, Cn, seed, n_frames) for (W, H, Cn, seed) in STREAMS]
    alone = [_alone(fr, seed) for fr, (_, _, _, seed) in zip(data, STREAMS)]
    # a budget that holds the two largest streams (and their share of the batch work area) only
    need = sorted(lib.lvbgs_device_bytes(L.ALGO_SUBSENSE, W, H, Cn, 50) + 32 * W * H for (W, H, Cn, _) in STREAMS)
    budget = need[-1] + need[-2] + 1024
    with serving.StreamServer(hbm_budget_bytes=budget, idle_spill_ms=0.0, max_queue=64) as srv:
        ids = [srv.open(fr[0], params={"seed": seed}) for fr, (_, _, _, seed) in zip(data, STREAMS)]
        masks = {}

        def submit(i, t):
            W, H = STREAMS[i][0], STREAMS[i][1]
            m = np.full((H, W), 77, np.uint8)
            masks[(i, t)] = m
            assert srv.submit(ids[i], data[i][t], m, tag=t)

        results = []
        # phase 1: five frames of every stream at once; two fit, the others wait for admission
        for t in range(1, 6):
            for i in range(len(STREAMS)):
                submit(i, t)
        srv.drain()
        results += srv.poll(4096)
        # phase 2: streams take turns, so that idle ones spill and come back
        order = [0, 2, 1, 3, 2, 0, 3, 1]
        for k, i in enumerate(order):
            for t in range(6 + (k // 4) * 3, 9 + (k // 4) * 3):
                submit(i, t)
            srv.drain()
            results += srv.poll(4096)
        # phase 3: the last frame of every stream, interleaved
        for i in (3, 1, 0, 2):
            submit(i, 12)
        srv.drain()
        results += srv.poll(4096)
        st = srv.stats()
        p50, p99 = srv.latency_quantile(0.5), srv.latency_quantile(0.99)
    assert all(r[2] == L.OK for r in results), [r for r in results if r[2] != L.OK][:3]
    assert len(results) == len(masks) == len(STREAMS) * (n_frames - 1)
    for (i, t), m in masks.items():
        diff = int((m != alone[i][t - 1]).sum())
        assert diff == 0, "stream %d frame %d: served mask differs from the stream alone at %d px" % (i, t, diff)
    assert st["spills"] > 0 and st["restores"] > 0, st
    assert st["admitted"] == len(STREAMS)
    assert st["peak_device_bytes"] <= budget
    assert 0 < p50 <= p99


@pytest.mark.gpu
def test_queue_limit_and_unknown_streams():
    data = _frames(64, 48, 3, 21, 4)
    with serving.StreamServer(max_queue=2) as srv:
        sid = srv.open(data[0])
        mask = [np.zeros((48, 64), np.uint8) for _ in range(3)]
        accepted = [srv.submit(sid, data[1 + k], mask[k], tag=k) for k in range(3)]
        # the stream may already have started its first frame, so two or three are accepted
        assert accepted[0] and accepted[1]
        srv.drain()
        res = srv.poll(16)
        assert len(res) == sum(accepted) and all(r[2] == L.OK for r in res)
        with pytest.raises(Exception):
            srv.submit(sid + 100, data[1], mask[0])
        srv.close(sid)
        srv.drain()
        assert srv.stream_state(sid) == "closed"


@pytest.mark.gpu
def test_serving_workload_simulation_short():
    r = serving.simulate(duration_s=3.0, warmup_s=1.0, arrival_rate=3.0, life_min_s=1.0, life_max_s=3.0,
                         res_prob=[0.7, 0.3, 0.0, 0.0], pool_frames=2, render_threads=2, seed=3)
    assert r["status"] == 0
    assert r["frames"] > 0 and r["mpix_per_s"] > 0
    assert 0 < r["p50_ms"] <= r["p99_ms"] <= r["max_ms"]
    assert r["admitted"] >= 1 and r["ticks"] >= 1
    assert r["dropped"] == 0


@pytest.mark.gpu
def test_pawcs_and_subsense_streams_served_together_equal_alone():
    # SuBSENSE/PAWCS mixed: PAWCS frames run on the PAWCS lanes beside the batched SuBSENSE ticks;
    # every mask must equal the same stream run alone
    from litiv_gb300 import BackgroundSubtractorPAWCS
    mix = [(L.ALGO_SUBSENSE, 96, 64, 3, 31), (L.ALGO_PAWCS, 96, 72, 1, 32), (L.ALGO_SUBSENSE, 64, 48, 1, 33),
           (L.ALGO_PAWCS, 160, 120, 3, 34)]
    n_frames = 10
    data = [_frames(W, H, Cn, seed, n_frames) for (_, W, H, Cn, seed) in mix]
    alone = []
    for (algo, _, _, _, seed), fr in zip(mix, data):
        if algo == L.ALGO_PAWCS:
            b = BackgroundSubtractorPAWCS(seed=seed)
            b.initialize(fr[0])
            alone.append([b.apply(f) for f in fr[1:]])
        else:
            alone.append(_alone(fr, seed))
    with serving.StreamServer(max_queue=64, pawcs_lanes=2) as srv:
        ids = [srv.open(fr[0], params={"seed": seed}, algo=algo) for fr, (algo, _, _, _, seed) in zip(data, mix)]
        masks = {}
        for t in range(1, n_frames):
            for i, (_, W, H, _, _) in enumerate(mix):
                m = np.full((H, W), 77, np.uint8)
                masks[(i, t)] = m
                assert srv.submit(ids[i], data[i][t], m, tag=t)
        srv.drain()
        results = srv.poll(4096)
        st = srv.stats()
    assert all(r[2] == L.OK for r in results), [r for r in results if r[2] != L.OK][:3]
    assert len(results) == len(masks)
    for (i, t), m in masks.items():
        diff = int((m != alone[i][t - 1]).sum())
        assert diff == 0, "stream %d frame %d: served mask differs from the stream alone at %d px" % (i, t, diff)
    assert st["pawcs_frames"] == 2 * (n_frames - 1)



@pytest.mark.gpu
def test_pawcs_streams_spill_and_come_back_equal_alone():
    # two PAWCS streams under a budget that holds one of them at a time: they take turns, so the
    # idle one spills to pinned host memory (claimed from the PAWCS lanes first) and is restored when
    # its next frames arrive; every mask must equal the same stream run alone
    from litiv_gb300 import BackgroundSubtractorPAWCS
    lib = L.lib()
    mix = [(96, 72, 1, 41), (160, 120, 3, 42)]
    n_frames = 13
    data = [_frames(W, H, Cn, seed, n_frames) for (W, H, Cn, seed) in mix]
    alone = []
    for (_, _, _, seed), fr in zip(mix, data):
        b = BackgroundSubtractorPAWCS(seed=seed)
        b.initialize(fr[0])
        alone.append([b.apply(f) for f in fr[1:]])
    need = [lib.lvbgs_device_bytes(L.ALGO_PAWCS, W, H, Cn, 50) + 32 * W * H for (W, H, Cn, _) in mix]
    budget = max(need) + 1024
    assert sum(need) > budget
    with serving.StreamServer(hbm_budget_bytes=budget, idle_spill_ms=0.0, max_queue=64, pawcs_lanes=1) as srv:
        ids = [srv.open(fr[0], params={"seed": seed}, algo=L.ALGO_PAWCS) for fr, (_, _, _, seed) in zip(data, mix)]
        masks = {}
        results = []
        for k, i in enumerate([0, 1, 0, 1]):
            for t in range(1 + (k // 2) * 6, 7 + (k // 2) * 6):
                W, H = mix[i][0], mix[i][1]
                m = np.full((H, W), 77, np.uint8)
                masks[(i, t)] = m
                assert srv.submit(ids[i], data[i][t], m, tag=t)
            srv.drain()
            results += srv.poll(4096)
        st = srv.stats()
    assert all(r[2] == L.OK for r in results), [r for r in results if r[2] != L.OK][:3]
    assert len(results) == len(masks) == 2 * (n_frames - 1)
    for (i, t), m in masks.items():
        diff = int((m != alone[i][t - 1]).sum())
        assert diff == 0, "stream %d frame %d: served mask differs from the stream alone at %d px" % (i, t, diff)
    assert st["spills"] > 0 and st["restores"] > 0, st
    assert st["peak_device_bytes"] <= budget
