"""Serving loop for many background-subtraction streams on one GPU (include/lvserve.h).

``StreamServer`` wraps the native scheduler: streams are admitted by their device bytes, the frames
that arrive while ticks run are batched into the next tick, idle streams spill to pinned host
memory, and every frame's latency (submission to mask in host memory) is recorded. ``simulate``
runs the serving workload (Poisson stream arrivals, 30 fps per stream, mixed resolutions) in the
native simulator and returns its throughput and latency figures.
"""
import ctypes as C

import numpy as np

from . import _lib as L
from .bgs import LvException

STATE_NAMES = {0: "resident", 1: "waiting", 2: "spilled", 3: "closed"}


def _check(st, srv=None, what="serving call"):
    if st != L.OK:
        msg = L.lib().lvserve_last_error(srv).decode(errors="replace") if srv else ""
        name = L.STATUS_NAMES[st] if 0 <= st < len(L.STATUS_NAMES) else str(st)
        raise LvException(st, "%s failed: %s %s" % (what, name, msg))


def default_config(**overrides):
    cfg = L.ServeConfig()
    L.lib().lvserve_default_config(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


class StreamServer:
    """A serving loop on one device. ``submit`` is non-blocking; ``poll`` returns finished frames.

    The numpy image and mask of a submitted frame are kept alive here until its result is polled.
    """

    def __init__(self, **config):
        self._lib = L.lib()
        self.config = default_config(**config)
        h = C.c_void_p()
        _check(self._lib.lvserve_create(C.byref(self.config), C.byref(h)), None, "lvserve_create")
        self._h = h
        self._keep = {}

    def open(self, init_image, params=None, roi=None, algo=L.ALGO_SUBSENSE):
        img = np.ascontiguousarray(init_image, dtype=np.uint8)
        H, W = img.shape[:2]
        Cn = 1 if img.ndim == 2 else img.shape[2]
        p = None
        if params is not None:
            p = L.LvbgsParams()
            self._lib.lvbgs_default_params(algo, C.byref(p))
            for k, v in params.items():
                setattr(p, k, v)
        r = None if roi is None else np.ascontiguousarray(roi, dtype=np.uint8)
        sid = C.c_int(-1)
        st = self._lib.lvserve_open(self._h, algo, C.byref(p) if p is not None else None,
                                    img.ctypes.data_as(C.c_void_p), W, H, Cn, 0,
                                    r.ctypes.data_as(C.c_void_p) if r is not None else None, C.byref(sid))
        _check(st, self._h, "lvserve_open")
        return sid.value

    def submit(self, stream_id, image, mask, learning_rate=0.0, tag=0):
        """Queues one frame; returns False (frame not queued) when the stream's queue is full."""
        img = np.ascontiguousarray(image, dtype=np.uint8)
        if mask.dtype != np.uint8 or not mask.flags.c_contiguous:
            raise ValueError("mask must be a C-contiguous uint8 array")
        st = self._lib.lvserve_submit(self._h, int(stream_id), img.ctypes.data_as(C.c_void_p), 0,
                                      mask.ctypes.data_as(C.c_void_p), float(learning_rate), int(tag))
        if st == L.BUSY:
            return False
        _check(st, self._h, "lvserve_submit")
        self._keep[(int(stream_id), int(tag))] = (img, mask)
        return True

    def close(self, stream_id):
        _check(self._lib.lvserve_close(self._h, int(stream_id)), self._h, "lvserve_close")

    def poll(self, max_results=1024, timeout_ms=0):
        buf = (L.ServeResult * max_results)()
        n = self._lib.lvserve_poll(self._h, buf, max_results, int(timeout_ms))
        out = []
        for i in range(n):
            r = buf[i]
            self._keep.pop((r.stream_id, r.tag), None)
            out.append((r.stream_id, r.tag, r.status, r.latency_ms))
        return out

    def drain(self, timeout_ms=120000):
        _check(self._lib.lvserve_drain(self._h, int(timeout_ms)), self._h, "lvserve_drain")

    def stats(self):
        s = L.ServeStats()
        _check(self._lib.lvserve_get_stats(self._h, C.byref(s)), self._h, "lvserve_get_stats")
        return {name: getattr(s, name) for name, _ in L.ServeStats._fields_}

    def latency_quantile(self, q):
        return self._lib.lvserve_latency_quantile(self._h, float(q))

    def stream_state(self, stream_id):
        return STATE_NAMES[self._lib.lvserve_stream_state(self._h, int(stream_id))]

    def destroy(self):
        if self._h:
            self._lib.lvserve_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def plan_room(used, budget, need, cand_bytes, cand_idle_ms, idle_spill_ms):
    """The scheduler's spill choice: indices of the candidates to spill, or None if the need cannot fit."""
    n = len(cand_bytes)
    b = (C.c_size_t * max(n, 1))(*cand_bytes)
    i = (C.c_double * max(n, 1))(*cand_idle_ms)
    out = (C.c_int * max(n, 1))()
    k = L.lib().lvserve_plan_room(used, budget, need, b, i, n, float(idle_spill_ms), out)
    return None if k < 0 else [out[j] for j in range(k)]


def default_sim_config(**overrides):
    cfg = L.SimConfig()
    L.lib().lvserve_default_sim_config(C.byref(cfg))
    for k, v in overrides.items():
        if k == "res_prob":
            for j, p in enumerate(v):
                cfg.res_prob[j] = p
        else:
            setattr(cfg, k, v)
    return cfg


def simulate(server=None, **sim):
    """Runs the serving workload; ``server`` holds lvserve_config overrides. Returns a dict."""
    scfg = default_config(**(server or {}))
    cfg = default_sim_config(**sim)
    res = L.SimResult()
    _check(L.lib().lvserve_simulate(C.byref(scfg), C.byref(cfg), C.byref(res)), None, "lvserve_simulate")
    return {name: getattr(res, name) for name, _ in L.SimResult._fields_}
