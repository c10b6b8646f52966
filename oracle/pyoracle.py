"""ORACLE (test infrastructure only): ctypes wrapper of oracle/_build/liboracle.so (the C
restatement of the reference's SuBSENSE, PAWCS, LOBSTER, ViBe and PBAS, "port") and of oracle/_ref/libref.so (the reference's own SuBSENSE /
PAWCS sources compiled against the project-written OpenCV stand-in, "reference"; built only where
the reference sources are present, see oracle/refshim/build_ref.py). Both expose the same C API,
so OracleSuBSENSE / OraclePAWCS drive either one (``impl=``).

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

MAP_NAMES = ["R", "V", "T", "DLAST", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST",
             "UNSTABLE", "BLINKS", "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL_INV", "LAST_RAW_BLINK", "ROI",
             "LAST_COLOR", "LAST_DESC", "SAMPLE_COLOR", "SAMPLE_DESC", "DS_LT", "DS_ST", "LUT"]


class OParams(C.Structure):
    _fields_ = [("desc_dist_threshold_offset", C.c_size_t), ("min_color_dist_threshold", C.c_size_t),
                ("bg_samples", C.c_size_t), ("required_bg_samples", C.c_size_t),
                ("samples_for_moving_avgs", C.c_size_t), ("rel_lbsp_threshold", C.c_float),
                ("lbsp_threshold_offset", C.c_size_t), ("default_median_blur_kernel_size", C.c_int),
                ("seed", C.c_uint64)]


class OScalars(C.Structure):
    _fields_ = [("frame_idx", C.c_uint64), ("frames_since_last_reset", C.c_uint64),
                ("model_reset_cooldown", C.c_uint64), ("auto_model_reset_enabled", C.c_int32),
                ("learning_rate_scaling_enabled", C.c_int32), ("use_3x3_spread", C.c_int32),
                ("median_blur_kernel_size", C.c_int32), ("lr_lower_cap", C.c_float), ("lr_upper_cap", C.c_float),
                ("last_nonzero_desc_ratio", C.c_float), ("nonzero_desc_count", C.c_uint64),
                ("tot_color_diff", C.c_uint64), ("n_relevant_px", C.c_uint64), ("orig_roi_px", C.c_uint64),
                ("stat_samples_evaluated", C.c_uint64), ("stat_sample_writes", C.c_uint64)]


PAWCS_MAP_NAMES = ["R", "V", "T", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST", "ILLUM", "UNSTABLE",
                   "BLINKS", "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL", "LAST_RAW_BLINK", "ROI", "LAST_COLOR",
                   "LAST_DESC", "DS_LT", "DS_ST", "LUT", "LW_COLOR", "LW_DESC", "LW_OCC", "LW_FIRST", "LW_LAST", "GW",
                   "GW_MAP", "GLUT"]


class PParams(C.Structure):
    _fields_ = [("desc_dist_threshold_offset", C.c_size_t), ("min_color_dist_threshold", C.c_size_t),
                ("max_words", C.c_size_t), ("samples_for_moving_avgs", C.c_size_t),
                ("rel_lbsp_threshold", C.c_float), ("lbsp_threshold_offset", C.c_size_t),
                ("default_median_blur_kernel_size", C.c_int), ("seed", C.c_uint64)]


class PScalars(C.Structure):
    _fields_ = [("frame_idx", C.c_uint64), ("frames_since_last_reset", C.c_uint64),
                ("model_reset_cooldown", C.c_uint64), ("lword_weight_offset", C.c_uint64),
                ("auto_model_reset_enabled", C.c_int32), ("using_moving_camera", C.c_int32),
                ("median_blur_kernel_size", C.c_int32), ("n_local_words", C.c_int32),
                ("n_global_words", C.c_int32), ("last_nonflat_ratio", C.c_float), ("n_relevant_px", C.c_uint64),
                ("orig_roi_px", C.c_uint64), ("ds_roi_px", C.c_uint64), ("stat_words_scanned", C.c_uint64),
                ("stat_gdict_events", C.c_uint64), ("stat_nb_updates", C.c_uint64)]


_lib = None
_ref_lib = None
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref.so")


class LParams(C.Structure):
    _fields_ = [("desc_dist_threshold", C.c_size_t), ("color_dist_threshold", C.c_size_t),
                ("bg_samples", C.c_size_t), ("required_bg_samples", C.c_size_t),
                ("rel_lbsp_threshold", C.c_float), ("lbsp_threshold_offset", C.c_size_t),
                ("default_median_blur_kernel_size", C.c_int), ("seed", C.c_uint64)]


class LScalars(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("n_relevant_px", C.c_uint64), ("orig_roi_px", C.c_uint64),
                ("stat_samples_evaluated", C.c_uint64), ("stat_sample_writes", C.c_uint64)]


LOBSTER_MAP_NAMES = ["LAST_FG", "ROI", "LAST_COLOR", "LAST_DESC", "SAMPLE_COLOR", "SAMPLE_DESC", "LUT"]


class BParams(C.Structure):
    _fields_ = [("color_dist_threshold", C.c_size_t), ("update_rate", C.c_float), ("bg_samples", C.c_size_t),
                ("required_bg_samples", C.c_size_t), ("seed", C.c_uint64)]


PBAS_MAP_NAMES = ["SAMPLE_COLOR", "SAMPLE_GRAD", "R", "T", "D", "GRAD"]


class VParams(C.Structure):
    _fields_ = [("color_dist_threshold", C.c_size_t), ("bg_samples", C.c_size_t),
                ("required_bg_samples", C.c_size_t), ("seed", C.c_uint64)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def build_reference(ref_root=None):
    """Builds oracle/_ref/libref.so from the reference's sources; returns its path, or None when the
    reference sources are not present."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("lv_build_ref", os.path.join(HERE, "refshim", "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(ref_root) if ref_root else mod.build()


def ref_lib():
    """The reference compiled from its own sources (None when it cannot be built here)."""
    global _ref_lib
    if _ref_lib is None:
        path = build_reference()
        if path is None and not os.path.exists(REF_LIB_PATH):
            return None
        L = C.CDLL(REF_LIB_PATH)
        for pre, Par, Sc in (("rsub_", OParams, OScalars), ("rpawcs_", PParams, PScalars), ("rlob_", LParams, LScalars)):
            getattr(L, pre + "create").restype = C.c_void_p
            getattr(L, pre + "create").argtypes = [C.POINTER(Par)]
            getattr(L, pre + "destroy").argtypes = [C.c_void_p]
            getattr(L, pre + "initialize").argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
            getattr(L, pre + "apply").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
            getattr(L, pre + "get_background").argtypes = [C.c_void_p, C.c_void_p]
            getattr(L, pre + "set_roi").argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
            getattr(L, pre + "get_background_descriptors").argtypes = [C.c_void_p, C.c_void_p]
            getattr(L, pre + "get_scalars").argtypes = [C.c_void_p, C.POINTER(Sc)]
            if pre != "rlob_":
                getattr(L, pre + "set_automatic_model_reset").argtypes = [C.c_void_p, C.c_int]
        L.r_last_error.restype = C.c_char_p
        L.rsub_refresh_model.argtypes = [C.c_void_p, C.c_float, C.c_int]
        L.rsub_map.restype = C.c_void_p
        L.rsub_map.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]
        L.rpawcs_refresh_model.argtypes = [C.c_void_p, C.c_size_t, C.c_float, C.c_int]
        L.rlob_refresh_model.argtypes = [C.c_void_p, C.c_float, C.c_int]
        L.rpbas_create.restype = C.c_void_p
        L.rpbas_create.argtypes = [C.POINTER(BParams)]
        L.rpbas_destroy.argtypes = [C.c_void_p]
        L.rpbas_initialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.rpbas_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.rpbas_get_background.argtypes = [C.c_void_p, C.c_void_p]
        L.rpbas_map.restype = C.c_void_p
        L.rpbas_map.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]
        L.rpbas_mean_grad.restype = C.c_float
        L.rpbas_mean_grad.argtypes = [C.c_void_p]
        L.rvibe_create.restype = C.c_void_p
        L.rvibe_create.argtypes = [C.POINTER(VParams)]
        L.rvibe_destroy.argtypes = [C.c_void_p]
        L.rvibe_initialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.rvibe_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.rvibe_get_background.argtypes = [C.c_void_p, C.c_void_p]
        L.rvibe_samples.restype = C.c_void_p
        L.rvibe_samples.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
        L.rlob_map.restype = C.c_void_p
        L.rlob_map.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]
        L.rpawcs_export.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
        L.rpawcs_export_bytes.restype = C.c_size_t
        L.rpawcs_export_bytes.argtypes = [C.c_void_p, C.c_int]
        _ref_lib = L
    return _ref_lib


class _Api:
    """Calls `name` of the restatement (prefix o...) or of the reference (prefix r...)."""

    def __init__(self, impl, port_prefix, ref_prefix):
        if impl == "port":
            self.L, self.pre = lib(), port_prefix
        elif impl == "reference":
            self.L, self.pre = ref_lib(), ref_prefix
            if self.L is None:
                raise RuntimeError("the reference cannot be built here (its sources are not present)")
        else:
            raise ValueError("impl must be 'port' or 'reference'")

    def __getattr__(self, name):
        return getattr(self.L, self.pre + name)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.osub_create.restype = C.c_void_p
        L.osub_create.argtypes = [C.POINTER(OParams)]
        L.osub_destroy.argtypes = [C.c_void_p]
        L.osub_initialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.osub_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.osub_refresh_model.argtypes = [C.c_void_p, C.c_float, C.c_int]
        L.osub_get_background.argtypes = [C.c_void_p, C.c_void_p]
        L.osub_set_roi.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.osub_get_background_descriptors.argtypes = [C.c_void_p, C.c_void_p]
        L.osub_set_automatic_model_reset.argtypes = [C.c_void_p, C.c_int]
        L.osub_map.restype = C.c_void_p
        L.osub_map.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]
        L.osub_get_scalars.argtypes = [C.c_void_p, C.POINTER(OScalars)]
        L.olbsp_compute2.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_long, C.c_float, C.c_size_t,
                                     C.c_void_p]
        L.osample_pos_7x7.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]
        L.oneighbor_pos.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]
        L.ophilox_block.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orun_pawcs_streams.restype = C.c_double
        L.orun_pawcs_streams.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_uint64), C.c_int]
        L.orun_streams.restype = C.c_double
        L.orun_streams.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_uint64), C.c_int,
                                   C.POINTER(C.c_void_p), C.c_int]
        L.opawcs_default_params.argtypes = [C.POINTER(PParams)]
        L.opawcs_create.restype = C.c_void_p
        L.opawcs_create.argtypes = [C.POINTER(PParams)]
        L.opawcs_destroy.argtypes = [C.c_void_p]
        L.opawcs_initialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.opawcs_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.opawcs_refresh_model.argtypes = [C.c_void_p, C.c_size_t, C.c_float, C.c_int]
        L.opawcs_get_background.argtypes = [C.c_void_p, C.c_void_p]
        L.opawcs_set_roi.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.opawcs_get_background_descriptors.argtypes = [C.c_void_p, C.c_void_p]
        L.opawcs_set_automatic_model_reset.argtypes = [C.c_void_p, C.c_int]
        L.opawcs_export.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]
        L.opawcs_export_bytes.restype = C.c_size_t
        L.opawcs_export_bytes.argtypes = [C.c_void_p, C.c_int]
        L.opawcs_get_scalars.argtypes = [C.c_void_p, C.POINTER(PScalars)]
        L.olob_default_params.argtypes = [C.POINTER(LParams)]
        L.olob_create.restype = C.c_void_p
        L.olob_create.argtypes = [C.POINTER(LParams)]
        L.olob_destroy.argtypes = [C.c_void_p]
        L.olob_initialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.olob_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.olob_refresh_model.argtypes = [C.c_void_p, C.c_float, C.c_int]
        L.olob_get_background.argtypes = [C.c_void_p, C.c_void_p]
        L.olob_get_background_descriptors.argtypes = [C.c_void_p, C.c_void_p]
        L.olob_map.restype = C.c_void_p
        L.olob_map.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]
        L.olob_get_scalars.argtypes = [C.c_void_p, C.POINTER(LScalars)]
        L.ovibe_default_params.argtypes = [C.POINTER(VParams)]
        L.ovibe_create.restype = C.c_void_p
        L.ovibe_create.argtypes = [C.POINTER(VParams)]
        L.ovibe_destroy.argtypes = [C.c_void_p]
        L.ovibe_initialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.ovibe_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.ovibe_get_background.argtypes = [C.c_void_p, C.c_void_p]
        L.ovibe_samples.restype = C.c_void_p
        L.ovibe_samples.argtypes = [C.c_void_p, C.POINTER(C.c_size_t)]
        L.ovibe_get_stats.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
        L.opbas_default_params.argtypes = [C.POINTER(BParams)]
        L.opbas_create.restype = C.c_void_p
        L.opbas_create.argtypes = [C.POINTER(BParams)]
        L.opbas_destroy.argtypes = [C.c_void_p]
        L.opbas_initialize.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.opbas_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.opbas_get_background.argtypes = [C.c_void_p, C.c_void_p]
        L.opbas_map.restype = C.c_void_p
        L.opbas_map.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]
        L.opbas_mean_grad.restype = C.c_float
        L.opbas_mean_grad.argtypes = [C.c_void_p]
        L.opbas_gradient.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orun_lobster_streams.restype = C.c_double
        L.orun_lobster_streams.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_uint64), C.c_int]
        _lib = L
    return _lib


class OracleSuBSENSE:
    """Sequential CPU SuBSENSE (the checker): the C restatement (impl="port") or the reference's own
    BackgroundSubtractorSuBSENSE (impl="reference")."""

    def __init__(self, seed=0, impl="port", **params):
        p = OParams()
        lib().osub_default_params(C.byref(p))
        p.seed = seed
        for k, v in params.items():
            setattr(p, k, v)
        self.params = p
        self.impl = impl
        self._a = _Api(impl, "osub_", "rsub_")
        self._o = self._a.create(C.byref(p))
        if not self._o:
            raise ValueError("invalid oracle parameters")
        self.shape = None

    def close(self):
        if self._o:
            self._a.destroy(self._o)
            self._o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self, img, roi=None):
        img = np.ascontiguousarray(img, np.uint8)
        H, W = img.shape[:2]
        Cc = img.shape[2] if img.ndim == 3 else 1
        r = None if roi is None else np.ascontiguousarray(roi, np.uint8)
        st = self._a.initialize(self._o, img.ctypes.data_as(C.c_void_p), W, H, Cc,
                                   r.ctypes.data_as(C.c_void_p) if r is not None else None)
        if st != 0:
            raise ValueError("oracle initialize failed (%d)" % st)
        self.shape = (H, W, Cc)

    def apply(self, img, lr=0.0):
        img = np.ascontiguousarray(img, np.uint8)
        H, W, _ = self.shape
        mask = np.empty((H, W), np.uint8)
        st = self._a.apply(self._o, img.ctypes.data_as(C.c_void_p), mask.ctypes.data_as(C.c_void_p), float(lr))
        if st != 0:
            raise ValueError("oracle apply failed (%d)%s" % (st, self._err()))
        return mask

    def _err(self):
        return ": " + ref_lib().r_last_error().decode(errors="replace") if self.impl == "reference" else ""

    def refresh_model(self, frac, force=False):
        return self._a.refresh_model(self._o, float(frac), 1 if force else 0)

    def set_automatic_model_reset(self, v):
        self._a.set_automatic_model_reset(self._o, 1 if v else 0)

    def background(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint8)
        self._a.get_background(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def set_roi(self, roi):
        r = np.ascontiguousarray(roi, dtype=np.uint8)
        if self._a.set_roi(self._o, r.ctypes.data_as(C.c_void_p), r.shape[1], r.shape[0]) != 0:
            raise ValueError("oracle setROI failed")

    def background_descriptors(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint16)
        self._a.get_background_descriptors(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def state_map(self, name):
        n = C.c_size_t()
        ptr = self._a.map(self._o, MAP_NAMES.index(name), C.byref(n))
        raw = np.ctypeslib.as_array((C.c_uint8 * n.value).from_address(ptr)).copy()
        H, W, Cc = self.shape
        from litiv_gb300.bgs import map_view  # layout helper only (pure numpy)
        return map_view(name, raw, W, H, Cc, self.params.bg_samples)

    def scalars(self):
        s = OScalars()
        self._a.get_scalars(self._o, C.byref(s))
        return {f: getattr(s, f) for f, _ in OScalars._fields_}


class OraclePAWCS:
    """Sequential CPU PAWCS (the checker): the C restatement (impl="port") or the reference's own
    BackgroundSubtractorPAWCS (impl="reference")."""

    def __init__(self, seed=0, impl="port", **params):
        p = PParams()
        lib().opawcs_default_params(C.byref(p))
        p.seed = seed
        for k, v in params.items():
            setattr(p, k, v)
        self.params = p
        self.impl = impl
        self._a = _Api(impl, "opawcs_", "rpawcs_")
        self._o = self._a.create(C.byref(p))
        if not self._o:
            raise ValueError("invalid oracle parameters")
        self.shape = None

    def close(self):
        if self._o:
            self._a.destroy(self._o)
            self._o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self, img, roi=None):
        img = np.ascontiguousarray(img, np.uint8)
        H, W = img.shape[:2]
        Cc = img.shape[2] if img.ndim == 3 else 1
        r = None if roi is None else np.ascontiguousarray(roi, np.uint8)
        st = self._a.initialize(self._o, img.ctypes.data_as(C.c_void_p), W, H, Cc,
                                     r.ctypes.data_as(C.c_void_p) if r is not None else None)
        if st != 0:
            raise ValueError("oracle initialize failed (%d)" % st)
        self.shape = (H, W, Cc)

    def apply(self, img, lr=0.0):
        img = np.ascontiguousarray(img, np.uint8)
        H, W, _ = self.shape
        mask = np.empty((H, W), np.uint8)
        st = self._a.apply(self._o, img.ctypes.data_as(C.c_void_p), mask.ctypes.data_as(C.c_void_p), float(lr))
        if st != 0:
            raise ValueError("oracle apply failed (%d)" % st)
        return mask

    def refresh_model(self, base_occ, occ_decr_frac, force=False):
        return self._a.refresh_model(self._o, int(base_occ), float(occ_decr_frac), 1 if force else 0)

    def set_automatic_model_reset(self, v):
        self._a.set_automatic_model_reset(self._o, 1 if v else 0)

    def background(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint8)
        self._a.get_background(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def set_roi(self, roi):
        r = np.ascontiguousarray(roi, dtype=np.uint8)
        if self._a.set_roi(self._o, r.ctypes.data_as(C.c_void_p), r.shape[1], r.shape[0]) != 0:
            raise ValueError("oracle setROI failed")

    def background_descriptors(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint16)
        self._a.get_background_descriptors(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def state_map(self, name):
        """Raw bytes of one exported state array (layouts in oracle.h, OPAWCS_MAP_*)."""
        which = PAWCS_MAP_NAMES.index(name)
        n = self._a.export_bytes(self._o, which)
        out = np.empty(n, np.uint8)
        st = self._a.export(self._o, which, out.ctypes.data_as(C.c_void_p), n)
        if st != 0:
            raise ValueError("oracle export failed (%d)" % st)
        return out

    def scalars(self):
        s = PScalars()
        self._a.get_scalars(self._o, C.byref(s))
        return {f: getattr(s, f) for f, _ in PScalars._fields_}


class OracleLOBSTER:
    """Sequential CPU LOBSTER (the checker): the C restatement (impl="port") or the reference's own
    BackgroundSubtractorLOBSTER (impl="reference"). apply()'s learning rate defaults to the reference's
    getDefaultLearningRate() (16)."""

    def __init__(self, seed=0, impl="port", **params):
        p = LParams()
        lib().olob_default_params(C.byref(p))
        p.seed = seed
        for k, v in params.items():
            setattr(p, k, v)
        self.params = p
        self.impl = impl
        self._a = _Api(impl, "olob_", "rlob_")
        self._o = self._a.create(C.byref(p))
        if not self._o:
            raise ValueError("invalid oracle parameters")
        self.shape = None

    def close(self):
        if self._o:
            self._a.destroy(self._o)
            self._o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self):
        return ": " + ref_lib().r_last_error().decode(errors="replace") if self.impl == "reference" else ""

    def initialize(self, img, roi=None):
        img = np.ascontiguousarray(img, np.uint8)
        H, W = img.shape[:2]
        Cc = img.shape[2] if img.ndim == 3 else 1
        r = None if roi is None else np.ascontiguousarray(roi, np.uint8)
        st = self._a.initialize(self._o, img.ctypes.data_as(C.c_void_p), W, H, Cc,
                                r.ctypes.data_as(C.c_void_p) if r is not None else None)
        if st != 0:
            raise ValueError("oracle initialize failed (%d)%s" % (st, self._err()))
        self.shape = (H, W, Cc)

    def apply(self, img, lr=16.0):
        img = np.ascontiguousarray(img, np.uint8)
        H, W, _ = self.shape
        mask = np.empty((H, W), np.uint8)
        st = self._a.apply(self._o, img.ctypes.data_as(C.c_void_p), mask.ctypes.data_as(C.c_void_p), float(lr))
        if st != 0:
            raise ValueError("oracle apply failed (%d)%s" % (st, self._err()))
        return mask

    def refresh_model(self, frac, force=False):
        return self._a.refresh_model(self._o, float(frac), 1 if force else 0)

    def background(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint8)
        self._a.get_background(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def background_descriptors(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint16)
        self._a.get_background_descriptors(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def state_map(self, name):
        """LAST_FG / ROI (uint8 [H, W]), LAST_COLOR (uint8 [H, W(, C)]), LAST_DESC (uint16 [H, W(, C)]),
        SAMPLE_COLOR (uint8 [N, H, W(, C)]), SAMPLE_DESC (uint16 [N, H, W(, C)]), LUT (uint8 [256])"""
        n = C.c_size_t()
        ptr = self._a.map(self._o, LOBSTER_MAP_NAMES.index(name), C.byref(n))
        raw = np.ctypeslib.as_array((C.c_uint8 * n.value).from_address(ptr)).copy()
        H, W, Cc = self.shape
        tail = (H, W, Cc) if Cc > 1 else (H, W)
        if name in ("LAST_FG", "ROI"):
            return raw.reshape(H, W)
        if name == "LUT":
            return raw
        if name == "LAST_COLOR":
            return raw.reshape(tail)
        if name == "LAST_DESC":
            return raw.view(np.uint16).reshape(tail)
        if name == "SAMPLE_COLOR":
            return raw.reshape((-1,) + tail)
        return raw.view(np.uint16).reshape((-1,) + tail)

    def scalars(self):
        s = LScalars()
        self._a.get_scalars(self._o, C.byref(s))
        return {f: getattr(s, f) for f, _ in LScalars._fields_}


class OracleViBe:
    """Sequential CPU ViBe (the checker): the C restatement (impl="port") or the reference's own
    BackgroundSubtractorViBe_1ch / _3ch (impl="reference"), chosen by the frame's channel count.
    apply()'s learning rate defaults to BGSVIBE_DEFAULT_LEARNING_RATE (16)."""

    def __init__(self, seed=0, impl="port", **params):
        p = VParams()
        lib().ovibe_default_params(C.byref(p))
        p.seed = seed
        for k, v in params.items():
            setattr(p, k, v)
        self.params = p
        self.impl = impl
        self._a = _Api(impl, "ovibe_", "rvibe_")
        self._o = self._a.create(C.byref(p))
        if not self._o:
            raise ValueError("invalid oracle parameters")
        self.shape = None

    def close(self):
        if self._o:
            self._a.destroy(self._o)
            self._o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self, img):
        img = np.ascontiguousarray(img, np.uint8)
        H, W = img.shape[:2]
        Cc = img.shape[2] if img.ndim == 3 else 1
        if self._a.initialize(self._o, img.ctypes.data_as(C.c_void_p), W, H, Cc) != 0:
            raise ValueError("oracle initialize failed")
        self.shape = (H, W, Cc)

    def apply(self, img, lr=16.0):
        img = np.ascontiguousarray(img, np.uint8)
        H, W, _ = self.shape
        mask = np.empty((H, W), np.uint8)
        if self._a.apply(self._o, img.ctypes.data_as(C.c_void_p), mask.ctypes.data_as(C.c_void_p), float(lr)) != 0:
            raise ValueError("oracle apply failed")
        return mask

    def background(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint8)
        self._a.get_background(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def samples(self):
        """uint8 [N, H, W(, C)]"""
        n = C.c_size_t()
        ptr = self._a.samples(self._o, C.byref(n))
        raw = np.ctypeslib.as_array((C.c_uint8 * n.value).from_address(ptr)).copy()
        H, W, Cc = self.shape
        return raw.reshape((-1, H, W, Cc) if Cc > 1 else (-1, H, W))

    def stats(self):
        """apply() calls, samples evaluated, sample writes (the port only)"""
        out = (C.c_uint64 * 3)()
        lib().ovibe_get_stats(self._o, out)
        return list(out)


class OraclePBAS:
    """Sequential CPU PBAS (the checker): the C restatement (impl="port") or the reference's own
    BackgroundSubtractorPBAS_1ch / _3ch (impl="reference"), chosen by the frame's channel count.
    apply()'s learning rate override defaults to BGSPBAS_DEFAULT_LEARNING_RATE_OVERRIDE (-1: T(x))."""

    def __init__(self, seed=0, impl="port", **params):
        p = BParams()
        lib().opbas_default_params(C.byref(p))
        p.seed = seed
        for k, v in params.items():
            setattr(p, k, v)
        self.params = p
        self.impl = impl
        self._a = _Api(impl, "opbas_", "rpbas_")
        self._o = self._a.create(C.byref(p))
        if not self._o:
            raise ValueError("invalid oracle parameters")
        self.shape = None

    def close(self):
        if self._o:
            self._a.destroy(self._o)
            self._o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self, img):
        img = np.ascontiguousarray(img, np.uint8)
        H, W = img.shape[:2]
        Cc = img.shape[2] if img.ndim == 3 else 1
        if self._a.initialize(self._o, img.ctypes.data_as(C.c_void_p), W, H, Cc) != 0:
            raise ValueError("oracle initialize failed")
        self.shape = (H, W, Cc)

    def apply(self, img, lr=-1.0):
        img = np.ascontiguousarray(img, np.uint8)
        H, W, _ = self.shape
        mask = np.empty((H, W), np.uint8)
        if self._a.apply(self._o, img.ctypes.data_as(C.c_void_p), mask.ctypes.data_as(C.c_void_p), float(lr)) != 0:
            raise ValueError("oracle apply failed")
        return mask

    def background(self):
        H, W, Cc = self.shape
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint8)
        self._a.get_background(self._o, out.ctypes.data_as(C.c_void_p))
        return out

    def state_map(self, name):
        """SAMPLE_COLOR / SAMPLE_GRAD (uint8 [N, H, W(, C)]), R / T / D (float32 [H, W]); GRAD (the
        port only: the last frame's gradient image)"""
        n = C.c_size_t()
        ptr = self._a.map(self._o, PBAS_MAP_NAMES.index(name), C.byref(n))
        raw = np.ctypeslib.as_array((C.c_uint8 * n.value).from_address(ptr)).copy()
        H, W, Cc = self.shape
        tail = (H, W, Cc) if Cc > 1 else (H, W)
        if name in ("R", "T", "D"):
            return raw.view(np.float32).reshape(H, W)
        if name == "GRAD":
            return raw.reshape(tail)
        return raw.reshape((-1,) + tail)

    def mean_grad(self):
        return self._a.mean_grad(self._o)


def pbas_gradient(img):
    """The port's gradient image of a frame (GaussianBlur 3x3, Scharr, convertScaleAbs, addWeighted)"""
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape[:2]
    Cc = img.shape[2] if img.ndim == 3 else 1
    out = np.empty(img.shape, np.uint8)
    lib().opbas_gradient(img.ctypes.data_as(C.c_void_p), W, H, Cc, out.ctypes.data_as(C.c_void_p))
    return out


def lbsp_compute2(img, abs_threshold=None, rel_threshold=0.333, offset=0, out=None):
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape[:2]
    Cc = img.shape[2] if img.ndim == 3 else 1
    if out is None:
        out = np.zeros(img.shape, np.uint16)
    thr = -1 if abs_threshold is None else int(abs_threshold)
    lib().olbsp_compute2(img.ctypes.data_as(C.c_void_p), W, H, Cc, thr, float(rel_threshold), int(offset),
                         out.ctypes.data_as(C.c_void_p))
    return out


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().ophilox_block(c, k, o)
    return list(o)


def run_streams(frames_list, seeds, n_threads, warm_frames=0):
    """CPU baseline: frames_list[i] is a uint8 array [F, H, W(, C)]; returns the wall seconds of the
    applied frames after the first warm_frames (applied untimed)."""
    n = len(frames_list)
    arrs = [np.ascontiguousarray(f) for f in frames_list]
    ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in arrs])
    nf = (C.c_int * n)(*[a.shape[0] for a in arrs])
    ws = (C.c_int * n)(*[a.shape[2] for a in arrs])
    hs = (C.c_int * n)(*[a.shape[1] for a in arrs])
    cs = (C.c_int * n)(*[(a.shape[3] if a.ndim == 4 else 1) for a in arrs])
    sd = (C.c_uint64 * n)(*seeds)
    return lib().orun_streams(n, ptrs, nf, ws, hs, cs, sd, int(n_threads), None, int(warm_frames))


def run_pawcs_streams(frames_list, seeds, n_threads):
    """PAWCS CPU baseline: frames_list[i] is uint8 [F, H, W]; returns wall seconds of the apply phase."""
    n = len(frames_list)
    arrs = [np.ascontiguousarray(f) for f in frames_list]
    ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in arrs])
    nf = (C.c_int * n)(*[a.shape[0] for a in arrs])
    ws = (C.c_int * n)(*[a.shape[2] for a in arrs])
    hs = (C.c_int * n)(*[a.shape[1] for a in arrs])
    cs = (C.c_int * n)(*[(a.shape[3] if a.ndim == 4 else 1) for a in arrs])
    sd = (C.c_uint64 * n)(*seeds)
    return lib().orun_pawcs_streams(n, ptrs, nf, ws, hs, cs, sd, int(n_threads))


def run_lobster_streams(frames_list, seeds, n_threads):
    """LOBSTER CPU baseline (learning rate 16): frames_list[i] is uint8 [F, H, W(, C)]; returns wall
    seconds of the apply phase."""
    n = len(frames_list)
    arrs = [np.ascontiguousarray(f) for f in frames_list]
    ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in arrs])
    nf = (C.c_int * n)(*[a.shape[0] for a in arrs])
    ws = (C.c_int * n)(*[a.shape[2] for a in arrs])
    hs = (C.c_int * n)(*[a.shape[1] for a in arrs])
    cs = (C.c_int * n)(*[(a.shape[3] if a.ndim == 4 else 1) for a in arrs])
    sd = (C.c_uint64 * n)(*seeds)
    return lib().orun_lobster_streams(n, ptrs, nf, ws, hs, cs, sd, int(n_threads))
