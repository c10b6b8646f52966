"""ctypes binding of ``liblvbgs.so`` (the C-ABI declared in include/lvbgs.h, lvbgs_synth.h and
lvserve.h).

The library is the only compute path: there is no CPU fallback. Loading fails loudly when the
in-tree build is missing (build it with ``python -m litiv_gb300.build`` or
``__graft_entry__.build()``).
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# LVBGS_LIB selects another build of the same library (e.g. to compare two builds side by side)
LIB_PATH = os.environ.get("LVBGS_LIB") or os.path.join(HERE, "_build", "liblvbgs.so")

# lvbgs_status
OK, BAD_ARG, BAD_SIZE, BAD_TYPE, NOT_INITIALIZED, OOM, DEVICE_TIMEOUT, DEVICE_ERROR, UNSUPPORTED, BUSY = range(10)
STATUS_NAMES = ["OK", "BAD_ARG", "BAD_SIZE", "BAD_TYPE", "NOT_INITIALIZED", "OOM", "DEVICE_TIMEOUT",
                "DEVICE_ERROR", "UNSUPPORTED", "BUSY"]
ALGO_SUBSENSE, ALGO_PAWCS, ALGO_LOBSTER, ALGO_VIBE, ALGO_PBAS = 0, 1, 2, 3, 4

# map ids (LVBGS_MAP_*)
MAP_NAMES = ["R", "V", "T", "DLAST", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST",
             "UNSTABLE", "BLINKS", "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL_INV", "LAST_RAW_BLINK", "ROI",
             "LAST_COLOR", "LAST_DESC", "SAMPLE_COLOR", "SAMPLE_DESC", "DS_LT", "DS_ST", "LUT",
             "SAMPLE_GRAD", "GRAD", "MEAN_GRAD"]
MAP_IDS = {n: i for i, n in enumerate(MAP_NAMES)}


class LvbgsParams(C.Structure):
    _fields_ = [("desc_dist_threshold_offset", C.c_size_t), ("min_color_dist_threshold", C.c_size_t),
                ("bg_samples", C.c_size_t), ("required_bg_samples", C.c_size_t),
                ("samples_for_moving_avgs", C.c_size_t), ("rel_lbsp_threshold", C.c_float),
                ("lbsp_threshold_offset", C.c_size_t), ("default_median_blur_kernel_size", C.c_int),
                ("seed", C.c_uint64), ("device_id", C.c_int), ("update_rate", C.c_float)]


class LvbgsFrame(C.Structure):
    _fields_ = [("image", C.c_void_p), ("stride", C.c_size_t), ("fgmask", C.c_void_p),
                ("learning_rate", C.c_double)]


class HostPackets(C.Structure):
    """lvbgs_host_packets: packets already in host memory, for lvbgs_precache_copy_loader"""
    _fields_ = [("base", C.c_void_p), ("packet_bytes", C.c_size_t), ("count", C.c_size_t)]


PACKET_LOADER = C.CFUNCTYPE(C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(C.c_uint8), C.c_size_t)


class LvbgsScalars(C.Structure):
    _fields_ = [("frame_idx", C.c_uint64), ("frames_since_last_reset", C.c_uint64),
                ("model_reset_cooldown", C.c_uint64), ("auto_model_reset_enabled", C.c_int32),
                ("learning_rate_scaling_enabled", C.c_int32), ("use_3x3_spread", C.c_int32),
                ("median_blur_kernel_size", C.c_int32), ("lr_lower_cap", C.c_float), ("lr_upper_cap", C.c_float),
                ("last_nonzero_desc_ratio", C.c_float), ("nonzero_desc_count", C.c_uint64),
                ("tot_color_diff", C.c_uint64), ("n_relevant_px", C.c_uint64), ("orig_roi_px", C.c_uint64),
                ("stat_samples_evaluated", C.c_uint64), ("stat_sample_writes", C.c_uint64),
                ("stat_repair_rounds", C.c_uint64), ("stat_repair_rematched", C.c_uint64)]


class SynthConfig(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("channels", C.c_int), ("seed", C.c_uint64),
                ("noise_sigma_milli", C.c_int), ("n_shapes", C.c_int), ("shape_min", C.c_int),
                ("shape_max", C.c_int), ("speed_min_q8", C.c_int), ("speed_max_q8", C.c_int),
                ("ellipses_only", C.c_int), ("ripple", C.c_int), ("drift", C.c_int), ("n_stopping", C.c_int),
                ("n_frames", C.c_int), ("thermal", C.c_int)]


class ServeConfig(C.Structure):
    _fields_ = [("device_id", C.c_int), ("hbm_budget_bytes", C.c_size_t), ("host_spill_budget_bytes", C.c_size_t),
                ("max_live", C.c_int), ("max_queue", C.c_int), ("idle_spill_ms", C.c_double),
                ("max_inflight", C.c_int), ("pawcs_lanes", C.c_int)]


class ServeResult(C.Structure):
    _fields_ = [("stream_id", C.c_int), ("tag", C.c_uint64), ("status", C.c_int), ("latency_ms", C.c_double)]


class ServeStats(C.Structure):
    _fields_ = [("frames_done", C.c_uint64), ("px_done", C.c_uint64), ("ticks", C.c_uint64),
                ("admitted", C.c_uint64), ("rejected", C.c_uint64), ("busy_refusals", C.c_uint64),
                ("spills", C.c_uint64), ("restores", C.c_uint64), ("closed", C.c_uint64), ("live", C.c_int),
                ("waiting", C.c_int), ("resident", C.c_int), ("spilled", C.c_int),
                ("device_bytes_in_use", C.c_size_t), ("peak_device_bytes", C.c_size_t),
                ("mean_tick_streams", C.c_double), ("busy_ms", C.c_double), ("pawcs_frames", C.c_uint64)]


class SimConfig(C.Structure):
    _fields_ = [("duration_s", C.c_double), ("warmup_s", C.c_double), ("arrival_rate", C.c_double),
                ("life_min_s", C.c_double), ("life_max_s", C.c_double), ("fps", C.c_double),
                ("res_prob", C.c_double * 4), ("gray_prob", C.c_double), ("pawcs_prob", C.c_double),
                ("prefill", C.c_int),
                ("pool_frames", C.c_int), ("render_threads", C.c_int), ("seed", C.c_uint64)]


class SimResult(C.Structure):
    _fields_ = [("window_s", C.c_double), ("frames", C.c_uint64), ("mpix_per_s", C.c_double),
                ("frames_per_s", C.c_double), ("offered_mpix_per_s", C.c_double), ("p50_ms", C.c_double),
                ("p90_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("admit_wait_p50_ms", C.c_double), ("admit_wait_p99_ms", C.c_double),
                ("pawcs_p50_ms", C.c_double), ("pawcs_p99_ms", C.c_double), ("pawcs_frames", C.c_uint64),
                ("subsense_p50_ms", C.c_double), ("subsense_p99_ms", C.c_double), ("mean_live", C.c_double),
                ("mean_resident", C.c_double), ("mean_tick_streams", C.c_double), ("gpu_busy_frac", C.c_double),
                ("ticks", C.c_uint64), ("arrivals", C.c_uint64), ("admitted", C.c_uint64),
                ("rejected", C.c_uint64), ("dropped", C.c_uint64), ("spills", C.c_uint64),
                ("restores", C.c_uint64), ("late_frames", C.c_uint64), ("peak_live", C.c_int),
                ("peak_device_bytes", C.c_size_t), ("status", C.c_int)]


class PawcsScalars(C.Structure):
    _fields_ = [("frame_idx", C.c_uint64), ("frames_since_last_reset", C.c_uint64),
                ("model_reset_cooldown", C.c_uint64), ("lword_weight_offset", C.c_uint64),
                ("auto_model_reset_enabled", C.c_int32), ("using_moving_camera", C.c_int32),
                ("median_blur_kernel_size", C.c_int32), ("n_local_words", C.c_int32),
                ("n_global_words", C.c_int32), ("last_nonflat_ratio", C.c_float), ("n_relevant_px", C.c_uint64),
                ("orig_roi_px", C.c_uint64), ("ds_roi_px", C.c_uint64), ("fixed_point_rounds", C.c_uint64)]


# PAWCS state maps (LVBGS_PAWCS_MAP_*), same order and layouts as the oracle's OPAWCS_MAP_*
PAWCS_MAP_NAMES = ["R", "V", "T", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST", "ILLUM", "UNSTABLE",
                   "BLINKS", "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL", "LAST_RAW_BLINK", "ROI", "LAST_COLOR",
                   "LAST_DESC", "DS_LT", "DS_ST", "LUT", "LW_COLOR", "LW_DESC", "LW_OCC", "LW_FIRST", "LW_LAST", "GW",
                   "GW_MAP", "GLUT"]

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "lvbgs_default_params": (C.c_int, [C.c_int, C.POINTER(LvbgsParams)]),
    "lvbgs_create": (C.c_int, [C.c_int, C.POINTER(LvbgsParams), C.POINTER(C.c_void_p)]),
    "lvbgs_destroy": (C.c_int, [C.c_void_p]),
    "lvbgs_initialize": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_size_t, C.c_void_p]),
    "lvbgs_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_double, C.c_void_p]),
    "lvbgs_batch_apply": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(LvbgsFrame), C.c_int, C.c_void_p]),
    "lvbgs_batch_wait": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_void_p]),
    "lvbgs_get_background": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lvbgs_get_background_descriptors": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lvbgs_refresh_model": (C.c_int, [C.c_void_p, C.c_float, C.c_int]),
    "lvbgs_set_automatic_model_reset": (C.c_int, [C.c_void_p, C.c_int]),
    "lvbgs_get_default_learning_rate": (C.c_double, [C.c_void_p]),
    "lvbgs_get_roi": (C.c_int, [C.c_void_p, C.c_void_p]),
    "lvbgs_get_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "lvbgs_state_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_size_t]),
    "lvbgs_spill": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lvbgs_restore": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "lvbgs_lbsp_compute2": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_long, C.c_float, C.c_size_t,
                                      C.c_void_p, C.c_int]),
    "lvbgs_lbsp_compute2_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_long, C.c_float,
                                              C.c_size_t, C.c_void_p, C.c_int, C.c_void_p]),
    "lvbgs_last_error": (C.c_char_p, [C.c_void_p]),
    "lvbgs_debug_map_bytes": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]),
    "lvbgs_debug_get_map": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "lvbgs_get_scalars": (C.c_int, [C.c_void_p, C.POINTER(LvbgsScalars)]),
    "lvbgs_debug_tick_profile": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int]),
    "lvbgs_debug_repair_phases": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int]),
    "lvbgs_debug_inject_fault": (C.c_int, [C.c_void_p, C.c_int]),
    "lvbgs_debug_pawcs_host_timing": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "lvbgs_classif_accumulate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                           C.POINTER(C.c_uint64), C.c_int, C.c_void_p]),
    "lvbgs_classif_metrics": (C.c_int, [C.POINTER(C.c_uint64), C.POINTER(C.c_double)]),
    "lvbgs_precacher_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]),
    "lvbgs_precacher_create_host": (C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]),
    "lvbgs_precacher_destroy": (C.c_int, [C.c_void_p]),
    "lvbgs_precacher_start": (C.c_int, [C.c_void_p, C.c_size_t]),
    "lvbgs_precacher_stop": (C.c_int, [C.c_void_p]),
    "lvbgs_precacher_get": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.POINTER(C.c_void_p),
                                      C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]),
    "lvbgs_precacher_is_active": (C.c_int, [C.c_void_p]),
    "lvbgs_precacher_last_index": (C.c_size_t, [C.c_void_p]),
    "lvbgs_precache_copy_loader": (C.c_size_t, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
    "lvbgs_set_roi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    "lvbgs_batch_set_repair_share": (C.c_int, [C.c_void_p, C.c_int]),
    "lvbgs_set_batch_groups": (C.c_int, [C.c_int]),
    "lvbgs_debug_set_timing": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "lvbgs_device_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_size_t]),
    "lvbgs_batch_create": (C.c_int, [C.c_int, C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]),
    "lvbgs_batch_destroy": (C.c_int, [C.c_void_p]),
    "lvbgs_batch_reserve": (C.c_int, [C.c_void_p, C.c_size_t, C.c_int]),
    "lvbgs_batch_submit": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(LvbgsFrame), C.c_int, C.c_void_p,
                                     C.POINTER(C.c_uint64)]),
    "lvbgs_batch_query": (C.c_int, [C.c_void_p, C.c_uint64]),
    "lvbgs_batch_complete": (C.c_int, [C.c_void_p, C.c_uint64]),
    "lvserve_default_config": (C.c_int, [C.POINTER(ServeConfig)]),
    "lvserve_create": (C.c_int, [C.POINTER(ServeConfig), C.POINTER(C.c_void_p)]),
    "lvserve_destroy": (C.c_int, [C.c_void_p]),
    "lvserve_open": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(LvbgsParams), C.c_void_p, C.c_int, C.c_int, C.c_int,
                               C.c_size_t, C.c_void_p, C.POINTER(C.c_int)]),
    "lvserve_submit": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_double, C.c_uint64]),
    "lvserve_close": (C.c_int, [C.c_void_p, C.c_int]),
    "lvserve_poll": (C.c_int, [C.c_void_p, C.POINTER(ServeResult), C.c_int, C.c_int]),
    "lvserve_drain": (C.c_int, [C.c_void_p, C.c_int]),
    "lvserve_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServeStats)]),
    "lvserve_latency_quantile": (C.c_double, [C.c_void_p, C.c_double]),
    "lvserve_reset_stats": (C.c_int, [C.c_void_p]),
    "lvserve_stream_state": (C.c_int, [C.c_void_p, C.c_int]),
    "lvserve_last_error": (C.c_char_p, [C.c_void_p]),
    "lvserve_plan_room": (C.c_int, [C.c_size_t, C.c_size_t, C.c_size_t, C.POINTER(C.c_size_t),
                                    C.POINTER(C.c_double), C.c_int, C.c_double, C.POINTER(C.c_int)]),
    "lvserve_default_sim_config": (C.c_int, [C.POINTER(SimConfig)]),
    "lvserve_simulate": (C.c_int, [C.POINTER(ServeConfig), C.POINTER(SimConfig), C.POINTER(SimResult)]),
    "lvbgs_pawcs_refresh_model": (C.c_int, [C.c_void_p, C.c_size_t, C.c_float, C.c_int]),
    "lvbgs_pawcs_get_scalars": (C.c_int, [C.c_void_p, C.POINTER(PawcsScalars)]),
    "lvbgs_pawcs_debug_export_bytes": (C.c_size_t, [C.c_void_p, C.c_int]),
    "lvbgs_pawcs_debug_export": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "lvsynth_preset": (C.c_int, [C.c_int, C.c_int, C.c_uint64, C.POINTER(SynthConfig)]),
    "lvsynth_create": (C.c_int, [C.POINTER(SynthConfig), C.POINTER(C.c_void_p)]),
    "lvsynth_destroy": (None, [C.c_void_p]),
    "lvsynth_render": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "lvsynth_render_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib = None


class LibraryMissing(ImportError):
    pass


def lib():
    """Returns the loaded library; raises LibraryMissing when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing("liblvbgs.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib
