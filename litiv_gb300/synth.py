"""Seeded synthetic video streams (include/lvbgs_synth.h) for tests and benchmarks."""
import ctypes as C

import numpy as np

from . import _lib as L


class SyntheticStream:
    """One seeded scene; ``render(t)`` gives (frame, ground truth) as numpy arrays."""

    def __init__(self, config=0, index=0, seed=1, **overrides):
        lib = L.lib()
        cfg = L.SynthConfig()
        st = lib.lvsynth_preset(config, index, seed, C.byref(cfg))
        if st != L.OK:
            raise ValueError("unknown synthetic preset %r/%r" % (config, index))
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self.cfg = cfg
        h = C.c_void_p()
        if lib.lvsynth_create(C.byref(cfg), C.byref(h)) != L.OK:
            raise ValueError("invalid synthetic configuration")
        self._h = h

    @property
    def shape(self):
        c = self.cfg
        return (c.height, c.width, c.channels) if c.channels > 1 else (c.height, c.width)

    @property
    def n_frames(self):
        return self.cfg.n_frames

    def render(self, t, with_gt=False):
        frame = np.empty(self.shape, np.uint8)
        gt = np.empty((self.cfg.height, self.cfg.width), np.uint8) if with_gt else None
        st = L.lib().lvsynth_render(self._h, int(t), frame.ctypes.data_as(C.c_void_p),
                                    gt.ctypes.data_as(C.c_void_p) if gt is not None else None)
        if st != L.OK:
            raise RuntimeError("render failed")
        return (frame, gt) if with_gt else frame

    def render_device(self, t, frame_ptr, gt_ptr=None, cuda_stream=None):
        st = L.lib().lvsynth_render_device(self._h, int(t), C.c_void_p(frame_ptr),
                                           C.c_void_p(gt_ptr) if gt_ptr else None,
                                           C.c_void_p(cuda_stream) if cuda_stream else None)
        if st != L.OK:
            raise RuntimeError("device render failed (%d)" % st)

    def close(self):
        if self._h:
            L.lib().lvsynth_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
