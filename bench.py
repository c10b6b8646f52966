"""Benchmark: SuBSENSE Mpix/s on the 64-stream mixed-resolution workload, batched vs plain.

A step is one frame tick of all 64 streams (16x320x240, 24x640x480, 16x1280x720, 8x1920x1080;
48 BGR + 16 grayscale; 39,936,000 pixels) processed by one batched frame step (15 kernel launches,
each over all streams). ``value`` is measured with the frames already resident in HBM; ``e2e`` goes through the
C-ABI (lvbgs_batch_apply) with pinned host frames and host masks, so the host->device frame copies
and device->host mask copies are inside the timed region. The plain form (one stream per launch,
64 launches per tick) is measured on the same frames. Inputs and model state (~24 GB) are far
larger than the 129 MB L2, so no flush is needed between steps.

``--impl reference`` times the CPU restatement of the reference (oracle/) on the host cores over a
bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SuBSENSE Mpix/s: batched 64-stream vs plain 1-stream on GB300; p99 frame ms"
# DRAM bytes (read + write) of the evaluation per pixel (lvbgs_k_eval + lvbgs_k_longscan), from an
# ncu capture of dram__bytes_read.sum + dram__bytes_write.sum on six streams of the mix (indices
# 52-57: four 1280x720, one of them gray, and two 1920x1080; 7,833,600 px): eval 878,392,064 +
# 393,505,536 bytes, long scans 435,291,392 + 44,822,016 bytes. roofline.traffic scales it to a tick
# by pixels.
EVAL_DRAM_BYTES_PER_PX = (878392064 + 393505536 + 435291392 + 44822016) / 7833600
WORKLOAD = ("subsense-mix64: 16x320x240 + 24x640x480 + 16x1280x720 + 8x1920x1080, 48 BGR + 16 gray, "
            "default parameters, synthetic seeded scenes")
# CPU sample: 4 streams of each resolution class
CPU_SAMPLE_STREAMS = [0, 1, 2, 3, 16, 17, 18, 19, 40, 41, 42, 43, 56, 57, 58, 59]


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        if not sm:
            return None
        srt = sorted(sm)
        return {"sm_mhz": srt[len(srt) // 2], "sm_min_mhz": srt[0], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(srt)}


KERNELS = ["eval", "longscan", "resolve", "repair", "commit", "runs", "vunion", "holes", "combine",
           "hcount", "median", "epilogue", "dilate", "reset", "close"]


def algorithmic_bytes(px_by_c):
    """Algorithmic HBM bytes of the whole path (per ROI pixel: frame c + mask 1 + 10 FP32 maps r+w 80 +
    last colour/descriptor r+w 6c + u8 maps r+w 12, plus 3c bytes per evaluated sample and per sample
    write)."""
    total = 0
    for c, (npx, s, w) in px_by_c.items():
        total += npx * (c + 1 + 80 + 6 * c + 12) + 3 * c * (s + w)
    return total


def eval_algorithmic_bytes(px_by_c):
    """Algorithmic bytes of the evaluation kernel alone (per ROI pixel: frame c + 8 FP32 maps r+w 64 +
    2 FP32 maps read 8 + last colour/descriptor r+w 6c + u8 maps 5, plus 3c bytes per evaluated sample)."""
    total = 0
    for c, (npx, s, w) in px_by_c.items():
        total += npx * (c + 64 + 8 + 6 * c + 5) + 3 * c * s
    return total


_CPU_FRAMES = {}


def cpu_baseline(n_frames=9, threads=None, warm_frames=3):
    """The oracle on the host cores: one instance per core across streams (lv::WorkerPool model). The
    first warm_frames applied frames run untimed, so that the timed frames start where the GPU's timed
    ticks start (frame 4 with the default 3 warm-up ticks)."""
    from litiv_gb300 import SyntheticStream
    from oracle import pyoracle
    import numpy as np
    threads = threads or os.cpu_count() or 1
    if n_frames not in _CPU_FRAMES:  # rendered once per process (the reference arm calls this per step)
        fr, px = [], 0
        for i in CPU_SAMPLE_STREAMS:
            s = SyntheticStream(3, index=i, seed=1)
            fr.append(np.stack([s.render(t) for t in range(n_frames)]))
            px += s.cfg.width * s.cfg.height * (n_frames - 1)
        _CPU_FRAMES[n_frames] = (fr, px)
    frames, px = _CPU_FRAMES[n_frames]
    seeds = [1000 + i for i in CPU_SAMPLE_STREAMS]
    px = px // (n_frames - 1) * (n_frames - 1 - warm_frames)
    wall = pyoracle.run_streams(frames, seeds, threads, warm_frames)
    return {"value": px / wall / 1e6, "unit": "Mpix/s", "cores": threads, "kind": "port",
            "sample": "%d streams of the mix (4 per resolution), frames %d-%d of each (after %d untimed), "
                      "%.1f Mpix in %.1f s" % (len(frames), 1 + warm_frames, n_frames - 1, warm_frames,
                                              px / 1e6, wall)}


def _runqueue_wait_ms():
    """Time the calling thread has spent waiting on a run queue (descheduled while runnable), from
    /proc/self/task/<tid>/schedstat; 0 where that is not available."""
    try:
        with open("/proc/self/task/%d/schedstat" % threading.get_native_id()) as f:
            return int(f.read().split()[1]) / 1e6
    except (OSError, ValueError, IndexError):
        return 0.0


def pawcs_run(n_frames, stream, cpu=True, channels=1):
    """PAWCS on the thermal-like 640x480 single-channel scene (channels=3: a 640x480 BGR scene of moving
    shapes on a smoothed texture): every frame through lvbgs_apply, from frames resident on the device
    (value) and from pinned host frames (e2e); wall clock per frame, since a PAWCS frame step waits for
    its fixed-point rounds. The first 10 frames are warm-up."""
    import ctypes as C
    import numpy as np
    import torch
    from litiv_gb300 import BackgroundSubtractorPAWCS, SyntheticStream
    from litiv_gb300 import _lib as L
    lib = L.lib()
    s = SyntheticStream(2, 0, 1) if channels == 1 else SyntheticStream(0, 0, 1, width=640, height=480, channels=3)
    W, H = s.cfg.width, s.cfg.height
    n = min(n_frames, s.n_frames)
    shp = (H, W) if channels == 1 else (H, W, 3)
    dev = torch.empty((n,) + shp, dtype=torch.uint8, device="cuda")
    for t in range(n):
        s.render_device(t, dev[t].data_ptr(), cuda_stream=stream.cuda_stream)
    host = torch.empty((n,) + shp, dtype=torch.uint8).pin_memory()
    host.copy_(dev.cpu())
    dmask = torch.empty((H, W), dtype=torch.uint8, device="cuda")
    hmask = torch.empty((H, W), dtype=torch.uint8).pin_memory()
    torch.cuda.synchronize()
    scene = ("640x480 single-channel thermal-like scene (six warm blobs, random walks)" if channels == 1 else
             "640x480 BGR scene (moving shapes on a smoothed texture, the SuBSENSE config 0 generator)")
    out = {"workload": "PAWCS, %s, default parameters, %d frames" % (scene, n)}
    for leg, frames, mask in (("device", dev, dmask), ("host", host, hmask)):
        b = BackgroundSubtractorPAWCS(seed=1)
        b.initialize(frames[0].cpu().numpy())
        ms, rounds, gpu_ev, waits, parts = [], [], [], [], []
        for t in range(1, n):
            # per frame: CUDA events around the frame step (its GPU time) and the calling thread's run-queue
            # wait (time spent descheduled), to tell a slow GPU step from a descheduled host thread
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            w0 = _runqueue_wait_ms()
            t0 = time.perf_counter()
            e0.record(stream)
            st = lib.lvbgs_apply(b.handle, C.c_void_p(frames[t].data_ptr()), 0, C.c_void_p(mask.data_ptr()), 0.0,
                                 C.c_void_p(stream.cuda_stream))
            e1.record(stream)
            ms.append((time.perf_counter() - t0) * 1e3)
            waits.append(_runqueue_wait_ms() - w0)
            gpu_ev.append((e0, e1))
            if st != L.OK:
                raise RuntimeError("PAWCS apply failed: %s" % lib.lvbgs_last_error(b.handle))
            hparts = (C.c_double * 5)()
            lib.lvbgs_debug_pawcs_host_timing(b.handle, hparts)
            parts.append([round(v, 2) for v in hparts])
            rounds.append(b.scalars()["fixed_point_rounds"])
        b.close()
        torch.cuda.synchronize()
        gms = [a.elapsed_time(z) for a, z in gpu_ev]
        m = np.array(ms[9:])
        med = float(np.percentile(m, 50))
        r = {"value": W * H / (m.mean() / 1e3) / 1e6, "unit": "Mpix/s", "frames_per_s": 1e3 / m.mean(),
             "ms_per_frame": float(m.mean()), "p50_frame_ms": med,
             # the same at the median frame time: the slow frames seen in some runs are pauses of 50-150 ms
             # inside single CUDA calls of the step (a launch, a wait or a copy; see slow_frames' parts),
             # with no throttle reason and the calling thread not descheduled
             "value_at_median_frame": W * H / (med / 1e3) / 1e6,
             "p99_frame_ms": float(np.percentile(m, 99)), "rounds_mean": float(np.mean(rounds)),
             "rounds_max": int(np.max(rounds)),
             # frames that took more than three times the median: index, wall ms, fixed-point rounds, GPU ms
             # between CUDA events around the step, ms the calling thread waited on the run queue, and the
             # host ms of the step's parts (lvbgs_debug_pawcs_host_timing: enqueue rounds, round waits,
             # enqueue the rest, final wait, status read)
             "slow_frames": [[t + 1, round(v, 2), int(rounds[t]), round(gms[t], 2), round(waits[t], 2), parts[t]]
                             for t, v in enumerate(ms) if t >= 9 and v > 3 * med],
             "median_frame_parts_ms": [round(float(np.median([q[i] for q in parts[9:]])), 3) for i in range(5)]}
        if leg == "device":
            out.update(r)
        else:
            r["h2d_bytes_per_step"] = W * H * channels
            r["d2h_bytes_per_step"] = W * H
            out["e2e"] = r
    if cpu:
        from oracle import pyoracle
        threads = os.cpu_count() or 1
        nf = 3
        fr, seeds = [], []
        for i in range(threads):
            si = (SyntheticStream(2, 0, 100 + i) if channels == 1 else
                  SyntheticStream(0, 0, 100 + i, width=640, height=480, channels=3))
            fr.append(np.stack([si.render(t) for t in range(nf)]))
            seeds.append(100 + i)
        wall = pyoracle.run_pawcs_streams(fr, seeds, threads)
        px = threads * (nf - 1) * W * H
        out["cpu_baseline"] = {"value": px / wall / 1e6, "unit": "Mpix/s", "cores": threads, "kind": "port",
                               "sample": "%d streams of the scene (one per core), %d applied frames each after "
                                         "initialization, %.1f Mpix in %.2f s" % (threads, nf - 1, px / 1e6, wall)}
    return out


def single_stream_run(config, n_frames, stream, cpu=True, cpu_frames=4):
    """SuBSENSE configs 0 and 1 of the benchmark (one seeded stream: 320x240 BGR, 200 frames; 1920x1080
    BGR, 500 frames): every frame through lvbgs_apply from frames resident on the device, wall clock
    per frame (the first 10 frames are warm-up); the CPU baseline is the oracle on one core (one
    instance per sequence, as the reference's apps run it) over the first cpu_frames frames."""
    import ctypes as C
    import numpy as np
    import torch
    from litiv_gb300 import BackgroundSubtractorSuBSENSE, SyntheticStream
    from litiv_gb300 import _lib as L
    lib = L.lib()
    s = SyntheticStream(config, 0, 1)
    W, H = s.cfg.width, s.cfg.height
    n = min(n_frames, s.n_frames)
    from litiv_gb300.metrics import BinClassif
    dev = torch.empty((n,) + s.shape, dtype=torch.uint8, device="cuda")
    dgt = torch.empty((n, H, W), dtype=torch.uint8, device="cuda")
    for t in range(n):
        s.render_device(t, dev[t].data_ptr(), dgt[t].data_ptr(), cuda_stream=stream.cuda_stream)
    dmask = torch.empty((H, W), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    b = BackgroundSubtractorSuBSENSE(seed=1)
    b.initialize(dev[0])
    ms = []
    quality = BinClassif()
    for t in range(1, n):
        t0 = time.perf_counter()
        st = lib.lvbgs_apply(b.handle, C.c_void_p(dev[t].data_ptr()), 0, C.c_void_p(dmask.data_ptr()), 0.0,
                             C.c_void_p(stream.cuda_stream))
        torch.cuda.current_stream().synchronize()
        stream.synchronize()
        ms.append((time.perf_counter() - t0) * 1e3)
        if st != L.OK:
            raise RuntimeError("apply failed: %s" % lib.lvbgs_last_error(b.handle))
        if t > 25:  # scored on the device after the timed call, once the model has learnt the scene
            quality.accumulate(dmask, dgt[t], cuda_stream=stream.cuda_stream)
    b.close()
    qm = quality.metrics()
    m = np.array(ms[9:])
    out = {"workload": "SuBSENSE config %d: one %dx%d %s stream, %d frames, default parameters" % (
               config, W, H, "BGR" if s.cfg.channels == 3 else "gray", n),
           "value": W * H / (m.mean() / 1e3) / 1e6, "unit": "Mpix/s", "frames_per_s": 1e3 / m.mean(),
           "ms_per_frame": float(m.mean()), "p50_frame_ms": float(np.percentile(m, 50)),
           "p99_frame_ms": float(np.percentile(m, 99)),
           "quality": {"f_measure": qm["dFMeasure"], "recall": qm["dRecall"], "precision": qm["dPrecision"],
                       "pbc": qm["dPBC"], "frames_scored": max(0, n - 26),
                       "note": "lv::BinClassif on the device (lvbgs_classif_accumulate) against the synthetic "
                               "ground truth (union of the shapes), frames 26 and later"}}
    if cpu:
        from oracle import pyoracle
        fr = np.stack([s.render(t) for t in range(cpu_frames + 1)])
        wall = pyoracle.run_streams([fr], [1], 1)
        px = W * H * cpu_frames
        out["cpu_baseline"] = {"value": px / wall / 1e6, "unit": "Mpix/s", "cores": 1, "kind": "port",
                               "sample": "the first %d applied frames on one core, %.1f Mpix in %.2f s" % (
                                   cpu_frames, px / 1e6, wall)}
    return out


SAMPLE_MODELS = {
    # name: (Python class, learning-rate argument of apply, the reference's default rate, description)
    "lobster": ("BackgroundSubtractorLOBSTER", 16.0, "LOBSTER (BackgroundSubtractorLOBSTER's non-parallel path)"),
    "vibe": ("BackgroundSubtractorViBe", 16.0, "ViBe (BackgroundSubtractorViBe_3ch)"),
    "pbas": ("BackgroundSubtractorPBAS", -1.0, "PBAS (BackgroundSubtractorPBAS_3ch, per-pixel update rates T(x))"),
}


def sample_model_run(algo, config, n_frames, stream, cpu=True, cpu_frames=4):
    """LOBSTER, ViBe or PBAS on the scenes of SuBSENSE configs 0 and 1 (one seeded stream: 320x240 BGR;
    1920x1080 BGR) at the reference's default learning rate: every frame through lvbgs_apply from frames
    resident on the device, wall clock per frame (the first 10 frames are warm-up); the CPU baseline is
    the oracle's restatement on one core over the first cpu_frames frames."""
    import ctypes as C
    import numpy as np
    import torch
    import litiv_gb300
    from litiv_gb300 import SyntheticStream
    from litiv_gb300 import _lib as L
    from litiv_gb300.metrics import BinClassif
    cls_name, lr, what = SAMPLE_MODELS[algo]
    lib = L.lib()
    s = SyntheticStream(config, 0, 1)
    W, H = s.cfg.width, s.cfg.height
    n = min(n_frames, s.n_frames)
    dev = torch.empty((n,) + s.shape, dtype=torch.uint8, device="cuda")
    dgt = torch.empty((n, H, W), dtype=torch.uint8, device="cuda")
    for t in range(n):
        s.render_device(t, dev[t].data_ptr(), dgt[t].data_ptr(), cuda_stream=stream.cuda_stream)
    dmask = torch.empty((H, W), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    b = getattr(litiv_gb300, cls_name)(seed=1)
    b.initialize(dev[0])
    ms = []
    quality = BinClassif()
    for t in range(1, n):
        t0 = time.perf_counter()
        st = lib.lvbgs_apply(b.handle, C.c_void_p(dev[t].data_ptr()), 0, C.c_void_p(dmask.data_ptr()), lr,
                             C.c_void_p(stream.cuda_stream))
        stream.synchronize()
        ms.append((time.perf_counter() - t0) * 1e3)
        if st != L.OK:
            raise RuntimeError("apply failed: %s" % lib.lvbgs_last_error(b.handle))
        if t > 25:
            quality.accumulate(dmask, dgt[t], cuda_stream=stream.cuda_stream)
    b.close()
    qm = quality.metrics()
    m = np.array(ms[9:])
    out = {"workload": "%s: one %dx%d %s stream (the SuBSENSE config %d scene), %d frames, default parameters, "
                       "learning rate %g" % (what, W, H, "BGR" if s.cfg.channels == 3 else "gray", config, n, lr),
           "value": W * H / (m.mean() / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_frame": float(m.mean()),
           "p50_frame_ms": float(np.percentile(m, 50)), "p99_frame_ms": float(np.percentile(m, 99)),
           "quality": {"f_measure": qm["dFMeasure"], "recall": qm["dRecall"], "precision": qm["dPrecision"],
                       "frames_scored": max(0, n - 26)}}
    if cpu:
        from oracle import pyoracle
        fr = np.stack([s.render(t) for t in range(cpu_frames + 1)])
        if algo == "lobster":
            wall = pyoracle.run_lobster_streams([fr], [1], 1)
        else:
            o = (pyoracle.OracleViBe if algo == "vibe" else pyoracle.OraclePBAS)(seed=1)
            o.initialize(fr[0])
            t0 = time.perf_counter()
            for t in range(1, cpu_frames + 1):
                o.apply(fr[t], lr)
            wall = time.perf_counter() - t0
        px = W * H * cpu_frames
        out["cpu_baseline"] = {"value": px / wall / 1e6, "unit": "Mpix/s", "cores": 1, "kind": "port",
                               "sample": "the first %d applied frames on one core, %.1f Mpix in %.2f s" % (
                                   cpu_frames, px / 1e6, wall)}
    return out


def sample_models_run(n_frames, stream, cpu=True):
    """the LOBSTER, ViBe and PBAS legs, each on the 320x240 and 1920x1080 scenes"""
    return {algo: {"config0": sample_model_run(algo, 0, n_frames, stream, cpu=cpu, cpu_frames=10),
                   "config1": sample_model_run(algo, 1, n_frames, stream, cpu=cpu, cpu_frames=2)}
            for algo in SAMPLE_MODELS}


def serving_subprocess(seconds, pawcs_lanes=1):
    """serving_run in a fresh child process (bench.py --serving-only); its JSON object, or a note of the
    failure."""
    cmd = [sys.executable, os.path.abspath(__file__), "--serving-only", "--serving-seconds", str(seconds),
           "--pawcs-lanes", str(pawcs_lanes)]
    try:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                           timeout=max(120.0, 6.0 * seconds + 60.0))
    except subprocess.TimeoutExpired:
        return {"status": -1, "note": "the serving run did not finish in time"}
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"status": -1, "note": "the serving run failed (exit %d): %s" % (r.returncode, r.stderr.strip()[-300:])}
    out = json.loads(lines[-1])
    out["process"] = "child process of its own"
    return out


def serving_run(seconds, pawcs_lanes=1):
    """The serving workload (Poisson arrivals of 4 streams/s up to 256 live, lives U[10, 60] s, 30 fps,
    320x240/640x480/1280x720/1920x1080 with p = .3/.3/.3/.1, a quarter single-channel), started from its
    stationary population, through the native serving loop with pinned host frames and masks."""
    from litiv_gb300 import serving
    r = serving.simulate(server={"pawcs_lanes": pawcs_lanes}, duration_s=seconds, warmup_s=3.0, render_threads=8, seed=1)
    keep = ["window_s", "frames", "mpix_per_s", "frames_per_s", "offered_mpix_per_s", "p50_ms", "p90_ms", "p99_ms",
            "max_ms", "admit_wait_p50_ms", "admit_wait_p99_ms", "subsense_p50_ms", "subsense_p99_ms", "pawcs_frames",
            "pawcs_p50_ms", "pawcs_p99_ms",
            "mean_live", "mean_resident", "mean_tick_streams", "gpu_busy_frac", "ticks", "arrivals", "admitted",
            "rejected", "dropped", "spills", "restores", "late_frames", "peak_live", "peak_device_bytes", "status"]
    out = {k: r[k] for k in keep}
    out["workload"] = ("SuBSENSE/PAWCS mixed: Poisson arrivals 4/s (max 256 live), lives U[10,60] s, 30 fps, "
                       "320x240/640x480/1280x720/1920x1080 at .3/.3/.3/.1, 1/4 single-channel, 2.5 %% of the streams "
                       "(either channel count) on PAWCS, frames of PAWCS streams on %d PAWCS lane(s) (lowest stream priority) "
                       "beside the batched SuBSENSE ticks; stationary start; latency = submit -> mask in pinned host "
                       "memory" % pawcs_lanes)
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(n_frames=6)
    t0 = time.time()
    for _ in range(args.steps):
        vals.append(cpu_baseline(n_frames=6))
    el = time.time() - t0
    v = sum(x["value"] for x in vals) / len(vals)
    cb = dict(vals[-1])
    cb["value"] = v
    out = {"metric": METRIC, "impl": "reference", "value": v, "unit": "Mpix/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/f32",
           "data": "synthetic", "config": {"workload": WORKLOAD, "sample": cb["sample"]},
           "cpu_baseline": cb, "e2e": {"value": v, "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--streams", type=int, default=64, help="number of streams of the mix (profiling: fewer)")
    ap.add_argument("--first", type=int, default=0, help="index of the first stream of the mix (profiling)")
    ap.add_argument("--plain-steps", type=int, default=5)
    ap.add_argument("--batch-groups", type=int, default=4,
                    help="concurrent groups a large batch is split into (lvbgs_set_batch_groups, 1..4)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--pawcs-frames", type=int, default=300,
                    help="frames of the PAWCS workload (640x480 thermal-like scene; 0: skip)")
    ap.add_argument("--serving-seconds", type=float, default=20.0,
                    help="measured span of the serving workload run (0: skip)")
    ap.add_argument("--pawcs-lanes", type=int, default=1,
                    help="host lanes running the PAWCS streams' frames in the serving run (lvserve_config.pawcs_lanes)")
    ap.add_argument("--serving-only", action="store_true",
                    help="run the serving workload alone and print its object (profiling)")
    ap.add_argument("--single-frames", type=int, default=100,
                    help="frames of the single-stream SuBSENSE configs 0 and 1 (0: skip)")
    ap.add_argument("--lobster-frames", type=int, default=100,
                    help="frames of the single-stream LOBSTER, ViBe and PBAS legs (0: skip)")
    ap.add_argument("--pawcs-channels", default="both", choices=["1", "3", "both"],
                    help="PAWCS legs: the single-channel scene (config 2), the BGR scene, or both")
    ap.add_argument("--pawcs-only", action="store_true",
                    help="run the PAWCS workload alone and print its object (profiling)")
    ap.add_argument("--lobster-only", action="store_true",
                    help="run the LOBSTER, ViBe and PBAS legs alone and print their object (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.pawcs_only:
        import torch
        torch.cuda.set_device(0)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        out = {}
        if args.pawcs_channels != "3":
            out = pawcs_run(args.pawcs_frames, stream, cpu=not args.no_cpu_baseline)
        if args.pawcs_channels != "1":
            out["bgr"] = pawcs_run(min(args.pawcs_frames, 100), stream, cpu=not args.no_cpu_baseline, channels=3)
        print(json.dumps(out))
        return

    if args.serving_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(serving_run(args.serving_seconds, args.pawcs_lanes)))
        return

    if args.lobster_only:
        import torch
        torch.cuda.set_device(0)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        print(json.dumps(sample_models_run(args.lobster_frames, stream, cpu=not args.no_cpu_baseline)))
        return

    import numpy as np
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    from litiv_gb300 import BackgroundSubtractorSuBSENSE, SyntheticStream
    from litiv_gb300 import _lib as L
    import ctypes as C

    lib = L.lib()
    n = args.streams
    prof_steps = 5  # ticks of the per-kernel profile pass (one group, after the timed region)
    ticks = 1 + args.warmup + args.steps + prof_steps
    synth = [SyntheticStream(3, index=args.first + i, seed=1) for i in range(n)]
    dev_frames = []  # per stream: uint8 tensor [ticks, H, W, C]
    for s in synth:
        shp = (ticks,) + s.shape
        buf = torch.empty(shp, dtype=torch.uint8, device="cuda")
        for t in range(ticks):
            s.render_device(t, buf[t].data_ptr(), None, torch.cuda.current_stream().cuda_stream)
        dev_frames.append(buf)
    torch.cuda.synchronize()
    px_step = sum(s.cfg.width * s.cfg.height for s in synth)
    # groups the library splits each tick into (lvbgs_batch_apply: >= 8 streams, >= 4 Mi px, >= 4 per group)
    groups = min(args.batch_groups, n // 4) if n >= 8 and px_step >= (4 << 20) else 1
    if lib.lvbgs_set_batch_groups(args.batch_groups) != 0:
        raise SystemExit("--batch-groups must be 1..4")
    # a dedicated stream: the library launches on it and the CUDA events are recorded on it (a NULL
    # stream pointer would mean "the handle's own stream" to the C-ABI)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = C.c_void_p(stream.cuda_stream)
    assert stream.cuda_stream != 0

    def make_subtractors(seed_base):
        subs = []
        for i, s in enumerate(synth):
            b = BackgroundSubtractorSuBSENSE(seed=seed_base + i, device_id=local)
            b.initialize(dev_frames[i][0])
            subs.append(b)
        return subs

    def frames_struct(subs, t, masks, host=None):
        fr = (L.LvbgsFrame * len(subs))()
        for i in range(len(subs)):
            fr[i].image = host[i][t].ctypes.data if host is not None else dev_frames[i][t].data_ptr()
            fr[i].stride = 0
            fr[i].fgmask = masks[i]
            fr[i].learning_rate = 0.0
        return fr

    def check(st, h):
        if st != L.OK:
            raise RuntimeError("lvbgs error %d: %s" % (st, lib.lvbgs_last_error(h)))

    # ---- batched form, device-resident frames ----
    subs = make_subtractors(1000)
    hs = (C.c_void_p * n)(*[b.handle for b in subs])
    dmasks = [torch.empty((s.cfg.height, s.cfg.width), dtype=torch.uint8, device="cuda") for s in synth]
    mptrs = [m.data_ptr() for m in dmasks]
    frs = [frames_struct(subs, t, mptrs) for t in range(ticks)]
    for t in range(1, 1 + args.warmup):
        check(lib.lvbgs_batch_apply(hs, frs[t], n, sptr), hs[0])
    check(lib.lvbgs_batch_wait(hs, n, sptr), hs[0])
    sc0 = [b.scalars() for b in subs]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clk:
        evs[0].record(stream)
        for k in range(args.steps):
            t = 1 + args.warmup + k
            check(lib.lvbgs_batch_apply(hs, frs[t], n, sptr), hs[0])
            evs[k + 1].record(stream)
        check(lib.lvbgs_batch_wait(hs, n, sptr), hs[0])
        torch.cuda.synchronize()
    tick_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    if world > 1:
        tt = torch.tensor([total_ms], dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(tt[0])
    sc1 = [b.scalars() for b in subs]
    value = px_step * args.steps * world / (total_ms / 1e3) / 1e6
    px_by_c = {}
    for s, a, b in zip(synth, sc0, sc1):
        c = s.cfg.channels
        e = px_by_c.setdefault(c, [0, 0, 0])
        e[0] += (b["frame_idx"] - a["frame_idx"]) * b["n_relevant_px"]
        e[1] += b["stat_samples_evaluated"] - a["stat_samples_evaluated"]
        e[2] += b["stat_sample_writes"] - a["stat_sample_writes"]
    alg_bytes_step = algorithmic_bytes({c: tuple(v) for c, v in px_by_c.items()}) / args.steps
    eval_bytes_step = eval_algorithmic_bytes({c: tuple(v) for c, v in px_by_c.items()}) / args.steps
    ms_step = total_ms / args.steps
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes_step / (ms_step / 1e3) / 1e9
    tick_sorted = sorted(tick_ms)
    p50 = tick_sorted[len(tick_sorted) // 2]
    p99 = tick_sorted[min(len(tick_sorted) - 1, int(round(0.99 * (len(tick_sorted) - 1))))]
    # per-kernel profile: a few more ticks run as one group (the timed ticks split large batches into
    # concurrent groups, whose kernels overlap), CUDA events around each kernel
    check(lib.lvbgs_set_batch_groups(1), None)
    check(lib.lvbgs_debug_set_timing(hs[0], 1, prof_steps), hs[0])
    pe = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    pe[0].record(stream)
    for k in range(prof_steps):
        check(lib.lvbgs_batch_apply(hs, frs[1 + args.warmup + args.steps + k], n, sptr), hs[0])
    pe[1].record(stream)
    check(lib.lvbgs_batch_wait(hs, n, sptr), hs[0])
    torch.cuda.synchronize()
    one_group_ms = pe[0].elapsed_time(pe[1]) / prof_steps
    check(lib.lvbgs_set_batch_groups(args.batch_groups), None)
    prof = (C.c_double * 16)()
    nprof = lib.lvbgs_debug_tick_profile(hs[0], 1, prof, 16)
    kernel_ms = {KERNELS[i]: round(prof[i], 4) for i in range(nprof)}
    lib.lvbgs_debug_set_timing(hs[0], 1, 0)
    ph = (C.c_double * 40)()
    nph = lib.lvbgs_debug_repair_phases(hs[0], 1, ph, 40)
    repair_phases = [round(ph[i], 1) for i in range(nph)]
    # the evaluation spans two kernels: the capped scan of every pixel, then the long scans
    eval_ms = sum(kernel_ms.get(k, 0.0) for k in ("eval", "longscan")) or float("nan")
    eval_achieved = eval_bytes_step / (eval_ms / 1e3) / 1e9
    rounds = sum(b["stat_repair_rounds"] - a["stat_repair_rounds"] for a, b in zip(sc0[:1], sc1[:1])) / args.steps
    remat = sum(b["stat_repair_rematched"] - a["stat_repair_rematched"] for a, b in zip(sc0, sc1)) / args.steps

    # ---- e2e through the C-ABI: host frames in, host masks out ----
    # Pipelined (the headline): a frame precacher over the pinned host ticks (lvbgs_precacher_create_host;
    # a packet is one tick, the 64 frames back to back) uploads each tick from pinned host memory on its
    # own copy stream while the previous tick computes; each tick then runs lvbgs_batch_apply on the
    # device copies, and the host waits for a tick's masks (two pinned mask sets, alternating) once the
    # next tick is enqueued, so that the mask download of one tick overlaps the next tick's kernels.
    # Precaching starts inside the timed region with an empty ring, so every timed tick's copies are
    # timed. Unpipelined (e2e.unpipelined): lvbgs_batch_apply on pinned host frames, uploads on the
    # compute stream, one wait per tick.
    e2e = None
    if not args.no_e2e:
        e2e_steps = args.steps
        h2d = sum(int(np.prod(s.shape)) for s in synth)
        offs, o = [], 0
        for s in synth:
            offs.append(o)
            o += (int(np.prod(s.shape)) + 255) // 256 * 256
        pkt_bytes = o
        first = 1 + args.warmup
        packets = torch.empty((e2e_steps, pkt_bytes), dtype=torch.uint8, pin_memory=True)
        for k in range(e2e_steps):
            for i in range(n):
                nb = int(np.prod(synth[i].shape))
                packets[k, offs[i]:offs[i] + nb].copy_(dev_frames[i][first + k].reshape(-1))
        hmasks = [[torch.empty((s.cfg.height, s.cfg.width), dtype=torch.uint8, pin_memory=True) for s in synth]
                  for _ in range(2)]
        hm2 = [[m.data_ptr() for m in ms] for ms in hmasks]
        hm = hm2[0]
        pc = C.c_void_p()
        check(lib.lvbgs_precacher_create_host(C.c_void_p(packets.data_ptr()), pkt_bytes, e2e_steps, local,
                                              C.byref(pc)), None)
        subs_e = make_subtractors(5000)
        hse = (C.c_void_p * n)(*[b.handle for b in subs_e])
        fr = (L.LvbgsFrame * n)()
        for t in range(1, first):  # warm-up ticks from device frames
            check(lib.lvbgs_batch_apply(hse, frames_struct(subs_e, t, hm), n, sptr), hse[0])
            check(lib.lvbgs_batch_wait(hse, n, sptr), hse[0])
        # the ring's pinned slots are allocated by a first start, outside the timed region
        check(lib.lvbgs_precacher_start(pc, 4 * pkt_bytes), None)
        check(lib.lvbgs_precacher_stop(pc), None)
        torch.cuda.synchronize()
        dp, hpp, sz = C.c_void_p(), C.c_void_p(), C.c_size_t()
        done = [torch.cuda.Event() for _ in range(e2e_steps)]
        t0 = time.perf_counter()
        check(lib.lvbgs_precacher_start(pc, 4 * pkt_bytes), None)
        for k in range(e2e_steps):
            check(lib.lvbgs_precacher_get(pc, k, sptr, C.byref(dp), C.byref(hpp), C.byref(sz)), None)
            for i in range(n):
                fr[i].image = dp.value + offs[i]
                fr[i].stride = 0
                fr[i].fgmask = hm2[k % 2][i]
                fr[i].learning_rate = 0.0
            check(lib.lvbgs_batch_apply(hse, fr, n, sptr), hse[0])
            done[k].record(stream)
            if k > 0:
                done[k - 1].synchronize()  # the previous tick's masks are on the host
        check(lib.lvbgs_batch_wait(hse, n, sptr), hse[0])  # the last tick's masks, and the device status
        el = time.perf_counter() - t0
        lib.lvbgs_precacher_destroy(pc)
        for b in subs_e:
            b.close()
        # unpipelined: pinned host frames straight into lvbgs_batch_apply
        subs_u = make_subtractors(5000)
        hsu = (C.c_void_p * n)(*[b.handle for b in subs_u])
        host = []
        for i in range(n):
            hb = torch.empty(dev_frames[i].shape, dtype=torch.uint8, pin_memory=True)
            hb.copy_(dev_frames[i])
            host.append(hb.numpy())
        fru = [frames_struct(subs_u, t, hm, host=host) for t in range(ticks)]
        for t in range(1, first):
            check(lib.lvbgs_batch_apply(hsu, fru[t], n, sptr), hsu[0])
        check(lib.lvbgs_batch_wait(hsu, n, sptr), hsu[0])
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for k in range(e2e_steps):
            check(lib.lvbgs_batch_apply(hsu, fru[first + k], n, sptr), hsu[0])
            check(lib.lvbgs_batch_wait(hsu, n, sptr), hsu[0])
        el_u = time.perf_counter() - t1
        for b in subs_u:
            b.close()
        e2e = {"value": px_step * e2e_steps / el / 1e6, "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": px_step, "ms_per_step": el / e2e_steps * 1e3,
               "note": "pinned host frames -> frame precacher (uploads on a copy stream overlapping the previous "
                       "tick, started inside the timed region) -> lvbgs_batch_apply -> host masks (two pinned sets; "
                       "the host waits for each tick's masks after enqueueing the next tick); wall clock",
               "unpipelined": {"value": px_step * e2e_steps / el_u / 1e6, "ms_per_step": el_u / e2e_steps * 1e3,
                               "note": "pinned host frames -> lvbgs_batch_apply (uploads on the compute "
                                       "stream) -> host masks"}}

    # ---- plain form: one stream per launch ----
    plain = None
    if args.plain_steps > 0:
        subs_p = make_subtractors(1000)
        for t in range(1, 1 + args.warmup):
            for i, b in enumerate(subs_p):
                one = (C.c_void_p * 1)(b.handle)
                check(lib.lvbgs_batch_apply(one, C.byref(frs[t][i]), 1, sptr), b.handle)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ps = min(args.plain_steps, args.steps)
        e0.record(stream)
        for k in range(ps):
            t = 1 + args.warmup + k
            for i, b in enumerate(subs_p):
                one = (C.c_void_p * 1)(b.handle)
                check(lib.lvbgs_batch_apply(one, C.byref(frs[t][i]), 1, sptr), b.handle)
        e1.record(stream)
        torch.cuda.synchronize()
        for b in subs_p:
            one = (C.c_void_p * 1)(b.handle)
            check(lib.lvbgs_batch_wait(one, 1, sptr), b.handle)
        pm = e0.elapsed_time(e1)
        plain = {"value": px_step * ps / (pm / 1e3) / 1e6, "unit": "Mpix/s", "ms_per_step": pm / ps,
                 "launches_per_step": n}
        for b in subs_p:
            b.close()

    # the serving workload runs in a child process of its own: it creates and frees hundreds of streams
    # (tens of GB of device memory and GBs of pinned host frames), and it is sensitive to the host
    # state the other legs leave (pinned buffers, caches); legs run right after it in the same process
    # showed pauses of 50-150 ms inside single CUDA calls
    serve = None
    if rank == 0 and args.serving_seconds > 0:
        with ClockSampler(local) as sclk:
            serve = serving_subprocess(args.serving_seconds, args.pawcs_lanes)
        if serve is not None:
            serve["clocks"] = sclk.summary()
    pawcs = None
    if rank == 0 and args.pawcs_frames > 0:
        with ClockSampler(local) as pclk:
            pawcs = pawcs_run(args.pawcs_frames, stream, cpu=not args.no_cpu_baseline)
        pawcs["clocks"] = pclk.summary()
        with ClockSampler(local) as pclk3:
            pawcs["bgr"] = pawcs_run(min(args.pawcs_frames, 100), stream, cpu=not args.no_cpu_baseline, channels=3)
        pawcs["bgr"]["clocks"] = pclk3.summary()
    singles = None
    if rank == 0 and args.single_frames > 0:
        singles = {"config0": single_stream_run(0, args.single_frames, stream, cpu=not args.no_cpu_baseline,
                                                cpu_frames=10),
                   "config1": single_stream_run(1, args.single_frames, stream, cpu=not args.no_cpu_baseline,
                                                cpu_frames=2)}

    models = {}
    if rank == 0 and args.lobster_frames > 0:
        models = sample_models_run(args.lobster_frames, stream, cpu=not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline()
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8/f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "streams": n, "px_per_step": px_step,
                       "l2": "inputs and model state (GBs) exceed L2; no flush",
                       "parallelism": "one batched frame step per tick: %d concurrent groups of about equal "
                                      "pixels, %d kernel launches each" % (groups, len(KERNELS))},
            "frames_per_s": n * args.steps * world / (total_ms / 1e3),
            "p50_frame_ms": p50, "p99_frame_ms": p99,
            "plain": plain,
            "batched_vs_plain": (value / world / plain["value"]) if plain else None,
            "roofline": {"bound": "hbm", "kernel": "lvbgs_k_eval + lvbgs_k_longscan",
                         "achieved": eval_achieved, "peak": peak,
                         "unit": "GB/s", "frac": eval_achieved / peak,
                         "traffic": EVAL_DRAM_BYTES_PER_PX * px_step, "traffic_per_px": EVAL_DRAM_BYTES_PER_PX,
                         "algorithmic_per_px": eval_bytes_step / px_step,
                         "note": "algorithmic bytes of the evaluation per tick / the summed average CUDA-event "
                                 "durations of its two kernels in the timed region; peak = measured copy "
                                 "bandwidth (of measured)"},
            "path_roofline": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                              "note": "algorithmic bytes of the whole frame step / tick time"},
            "repair": {"rounds_per_tick": rounds, "rematched_px_per_tick": remat,
                       "phases_us_last_tick": repair_phases},
            "kernel_ms": kernel_ms,
            "profile": {"ms_per_step_one_group": one_group_ms,
                        "note": "kernel_ms and roofline come from %d ticks run as one group with per-kernel CUDA "
                                "events; the timed ticks run large batches as %d concurrent groups of about equal "
                                "pixels (lvbgs_set_batch_groups)" % (prof_steps, groups)},
            "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": groups * len(KERNELS) * args.steps,
            "serving": serve,
            "pawcs": pawcs,
            "single_stream": singles,
            "lobster": models.get("lobster"),
            "vibe": models.get("vibe"),
            "pbas": models.get("pbas"),
            "clocks": clk.summary(),
        }
        print(json.dumps(out))
    for b in subs:
        b.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
