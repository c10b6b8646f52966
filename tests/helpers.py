"""Shared helpers of the parity tests: run the CUDA path and the oracle side by side."""
import numpy as np

FLOAT_MAPS = ["R", "V", "T", "DLAST", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST"]
U8_MAPS = ["UNSTABLE", "BLINKS", "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL_INV", "LAST_RAW_BLINK", "ROI"]
OTHER_MAPS = ["LAST_COLOR", "LAST_DESC", "SAMPLE_COLOR", "SAMPLE_DESC", "LUT"]
SCALARS = ["frame_idx", "frames_since_last_reset", "model_reset_cooldown", "auto_model_reset_enabled",
           "learning_rate_scaling_enabled", "use_3x3_spread", "median_blur_kernel_size", "lr_lower_cap",
           "lr_upper_cap", "last_nonzero_desc_ratio", "nonzero_desc_count", "tot_color_diff", "n_relevant_px",
           "orig_roi_px", "stat_samples_evaluated", "stat_sample_writes"]


def ulp_diff(a, b):
    ai = a.view(np.int32).astype(np.int64)
    bi = b.view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7fffffff), ai)
    bi = np.where(bi < 0, -(bi & 0x7fffffff), bi)
    return np.abs(ai - bi)


def compare_state(gpu, ora, with_samples=True, with_ds=True):
    """Returns a list of human-readable mismatches between the two models (empty when bit-exact)."""
    bad = []
    names = FLOAT_MAPS + U8_MAPS + OTHER_MAPS
    if with_ds and gpu.scalars()["learning_rate_scaling_enabled"]:
        names = names + ["DS_LT", "DS_ST"]
    for name in names:
        if not with_samples and name.startswith("SAMPLE"):
            continue
        g = gpu.state_map(name)
        o = ora.state_map(name)
        if g.dtype == np.float32:
            eq = g.view(np.uint32) == o.view(np.uint32)
        else:
            eq = g == o
        if not eq.all():
            idx = np.argwhere(~eq)
            first = tuple(int(v) for v in idx[0])
            extra = ""
            if g.dtype == np.float32:
                extra = " max ulp %d" % int(ulp_diff(g, o).max())
            bad.append("%s: %d differ, first at %s gpu=%r oracle=%r%s" % (
                name, int((~eq).sum()), first, g[first], o[first], extra))
    gs, os_ = gpu.scalars(), ora.scalars()
    for k in SCALARS:
        if gs[k] != os_[k]:
            bad.append("scalar %s: gpu=%r oracle=%r" % (k, gs[k], os_[k]))
    return bad
