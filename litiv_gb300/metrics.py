"""Change-detection evaluation on the device: lv::BinClassif and lv::BinClassifMetrics
(modules/datasets/include/litiv/datasets/metrics.hpp:32-66, 203-256) over the C-ABI."""
import ctypes as C

import numpy as np

from . import _lib as L

COUNTERS = ("nTP", "nTN", "nFP", "nFN", "nSE", "nDC")
METRICS = ("dRecall", "dSpecificity", "dFPR", "dFNR", "dPBC", "dPrecision", "dFMeasure", "dMCC")


def _ptr(a):
    """Host numpy array, or an object exposing a device pointer (data_ptr(), e.g. a torch tensor)."""
    if isinstance(a, np.ndarray):
        a = np.ascontiguousarray(a, np.uint8)
        return C.c_void_p(a.ctypes.data), a
    return C.c_void_p(a.data_ptr()), a


class BinClassif:
    """Classification counters of a binary classifier, accumulated on the device."""

    def __init__(self, device_id=0):
        self.counts = (C.c_uint64 * 6)()
        self.device_id = device_id

    def accumulate(self, mask, gt, roi=None, cuda_stream=None):
        """Adds the classification of mask (255 = positive) against CDnet-coded gt (and roi)."""
        H, W = mask.shape[:2]
        mp, k1 = _ptr(mask)
        gp, k2 = _ptr(gt) if gt is not None else (None, None)
        rp, k3 = _ptr(roi) if roi is not None else (None, None)
        st = L.lib().lvbgs_classif_accumulate(mp, gp, rp, W, H, self.counts, self.device_id,
                                              C.c_void_p(cuda_stream) if cuda_stream else None)
        if st != L.OK:
            raise RuntimeError("classification failed: %s" % L.lib().lvbgs_last_error(None))
        return self

    def as_dict(self):
        return {k: int(v) for k, v in zip(COUNTERS, self.counts)}

    def metrics(self):
        out = (C.c_double * 8)()
        L.lib().lvbgs_classif_metrics(self.counts, out)
        return {k: float(v) for k, v in zip(METRICS, out)}
