"""Host-side mirror of the reference's SuBSENSE interface, bound to the CUDA C-ABI.

``BackgroundSubtractorSuBSENSE`` mirrors ``BackgroundSubtractorSuBSENSE_`` of
modules/video/include/litiv/video/BackgroundSubtractorSuBSENSE.hpp:48-135 and the
``IIBackgroundSubtractor`` surface of BackgroundSubtractionUtils.hpp:24-97: same method names,
argument meaning and defaults; failures raise ``LvException`` as the reference's ``lvAssert_``
raises ``lv::Exception`` (modules/utils/include/litiv/utils/defines.hpp.in:111-113).
Images are numpy uint8 arrays [H,W] or [H,W,3] (or CUDA tensors exposing ``data_ptr()``).
"""
import ctypes as C

import numpy as np

from . import _lib as L


class LvException(RuntimeError):
    """Error raised by the library (the reference raises lv::Exception)."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (L.STATUS_NAMES[status] if 0 <= status < len(L.STATUS_NAMES) else status,
                                     message))
        self.status = status


def _check(st, handle=None):
    if st != L.OK:
        msg = L.lib().lvbgs_last_error(handle)
        raise LvException(st, msg.decode(errors="replace") if msg else "")


def _ptr(a):
    """(pointer, keepalive) of a numpy array or a CUDA tensor."""
    if a is None:
        return None, None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr()), a
    arr = np.ascontiguousarray(a)
    return C.c_void_p(arr.ctypes.data), arr


def _shape(img):
    shape = tuple(img.shape)
    if len(shape) == 2:
        return shape[0], shape[1], 1
    if len(shape) == 3:
        return shape[0], shape[1], shape[2]
    raise LvException(L.BAD_TYPE, "image must be [H,W] or [H,W,C]")


class BackgroundSubtractorSuBSENSE:
    """SuBSENSE on the GPU (the lv::CUDA specialisation the reference leaves missing)."""

    def __init__(self, nDescDistThresholdOffset=3, nMinColorDistThreshold=30, nBGSamples=50,
                 nRequiredBGSamples=2, nSamplesForMovingAvgs=100, fRelLBSPThreshold=0.333, seed=0,
                 device_id=0, nLBSPThresholdOffset=0, nDefaultMedianBlurKernelSize=9):
        lib = L.lib()
        p = L.LvbgsParams()
        _check(lib.lvbgs_default_params(L.ALGO_SUBSENSE, C.byref(p)))
        p.desc_dist_threshold_offset = nDescDistThresholdOffset
        p.min_color_dist_threshold = nMinColorDistThreshold
        p.bg_samples = nBGSamples
        p.required_bg_samples = nRequiredBGSamples
        p.samples_for_moving_avgs = nSamplesForMovingAvgs
        p.rel_lbsp_threshold = fRelLBSPThreshold
        p.lbsp_threshold_offset = nLBSPThresholdOffset
        p.default_median_blur_kernel_size = nDefaultMedianBlurKernelSize
        p.seed = seed
        p.device_id = device_id
        self.params = p
        h = C.c_void_p()
        _check(lib.lvbgs_create(L.ALGO_SUBSENSE, C.byref(p), C.byref(h)))
        self._h = h
        self._shape = None

    # -- lifetime --
    def close(self):
        if self._h:
            L.lib().lvbgs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- IIBackgroundSubtractor surface --
    def initialize(self, oInitImg, oROI=None):
        H, W, Cc = _shape(oInitImg)
        ip, keep = _ptr(oInitImg)
        rp, rkeep = _ptr(None if oROI is None else np.ascontiguousarray(oROI, dtype=np.uint8))
        _check(L.lib().lvbgs_initialize(self._h, ip, W, H, Cc, 0, rp), self._h)
        self._shape = (H, W, Cc)

    def apply(self, image, fgmask=None, learningRateOverride=0.0, stream=None):
        """apply(image, fgmask, learningRateOverride); `stream` (a cudaStream_t as int, or a
        torch.cuda.Stream) runs the frame step on that stream instead of the handle's own"""
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        if self._shape is None:
            raise LvException(L.NOT_INITIALIZED, "algo & model must be initialized first")
        H, W, Cc = _shape(image)
        if (H, W, Cc) != self._shape:
            raise LvException(L.BAD_SIZE, "input image type/size mismatch with initialization type/size")
        if fgmask is None:
            fgmask = np.empty((H, W), np.uint8)
        ip, keep = _ptr(image)
        mp, mkeep = _ptr(fgmask)
        _check(L.lib().lvbgs_apply(self._h, ip, 0, mp, float(learningRateOverride),
                                   C.c_void_p(stream) if stream else None), self._h)
        if isinstance(fgmask, np.ndarray) and mkeep is not fgmask:
            fgmask[...] = mkeep
        return fgmask

    def getBackgroundImage(self):
        H, W, Cc = self._need_init()
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint8)
        _check(L.lib().lvbgs_get_background(self._h, out.ctypes.data_as(C.c_void_p)), self._h)
        return out

    def getBackgroundDescriptorsImage(self):
        H, W, Cc = self._need_init()
        out = np.empty((H, W, Cc) if Cc > 1 else (H, W), np.uint16)
        _check(L.lib().lvbgs_get_background_descriptors(self._h, out.ctypes.data_as(C.c_void_p)), self._h)
        return out

    def refreshModel(self, fSamplesRefreshFrac, bForceFGUpdate=False):
        _check(L.lib().lvbgs_refresh_model(self._h, float(fSamplesRefreshFrac), 1 if bForceFGUpdate else 0), self._h)

    def setAutomaticModelReset(self, bVal):
        _check(L.lib().lvbgs_set_automatic_model_reset(self._h, 1 if bVal else 0), self._h)

    def getDefaultLearningRate(self):
        return L.lib().lvbgs_get_default_learning_rate(self._h)

    def getROICopy(self):
        H, W, _ = self._need_init()
        out = np.empty((H, W), np.uint8)
        _check(L.lib().lvbgs_get_roi(self._h, out.ctypes.data_as(C.c_void_p)), self._h)
        return out

    def validateROI(self, oROI):
        """validateROI (BackgroundSubtractionUtils.cpp:28-36): a copy of the 8UC1 ROI with its 2-pixel
        border ring (the LBSP pattern's reach) cleared."""
        r = np.array(oROI, dtype=np.uint8, copy=True)
        if r.ndim != 2 or r.size == 0:
            raise LvException(L.BAD_ARG, "provided ROI must be non-empty and of type 8UC1")
        r[:2, :] = 0
        r[-2:, :] = 0
        r[:, :2] = 0
        r[:, -2:] = 0
        return r

    def setROI(self, oROI):
        """setROI (BackgroundSubtractionUtils.cpp:38-48): on an initialized model, re-initializes it from
        the latest background image with the new ROI; otherwise keeps the ROI for initialize()."""
        r = np.ascontiguousarray(oROI, dtype=np.uint8)
        if r.ndim != 2 or r.size == 0:
            raise LvException(L.BAD_ARG, "provided ROI must be non-empty and of type 8UC1")
        _check(L.lib().lvbgs_set_roi(self._h, r.ctypes.data_as(C.c_void_p), r.shape[1], r.shape[0]), self._h)

    # -- lv::IParallelAlgo_<lv::CUDA> (modules/utils/include/litiv/utils/algo.hpp:82-129) --
    def isParallel(self):
        return True

    def getParallelAlgoType(self):
        return "CUDA"

    # -- serving helpers --
    def state_bytes(self):
        H, W, Cc = self._need_init()
        return L.lib().lvbgs_state_bytes(L.ALGO_SUBSENSE, W, H, Cc, self.params.bg_samples)

    def spill(self, host_buffer):
        """Moves the device state into host_buffer (a writable buffer of state_bytes() bytes)."""
        buf = (C.c_char * len(host_buffer)).from_buffer(host_buffer)
        _check(L.lib().lvbgs_spill(self._h, C.cast(buf, C.c_void_p), len(host_buffer)), self._h)

    def restore(self, host_buffer):
        buf = (C.c_char * len(host_buffer)).from_buffer(host_buffer)
        _check(L.lib().lvbgs_restore(self._h, C.cast(buf, C.c_void_p), len(host_buffer)), self._h)

    # -- inspection --
    def state_map(self, name):
        """A model map in the reference's layout (see include/lvbgs.h, LVBGS_MAP_*)."""
        H, W, Cc = self._need_init()
        mid = L.MAP_IDS[name]
        n = C.c_size_t()
        _check(L.lib().lvbgs_debug_map_bytes(self._h, mid, C.byref(n)), self._h)
        buf = np.empty(n.value, np.uint8)
        _check(L.lib().lvbgs_debug_get_map(self._h, mid, buf.ctypes.data_as(C.c_void_p), n.value), self._h)
        return map_view(name, buf, W, H, Cc, self.params.bg_samples)

    def scalars(self):
        s = L.LvbgsScalars()
        _check(L.lib().lvbgs_get_scalars(self._h, C.byref(s)), self._h)
        return {f: getattr(s, f) for f, _ in L.LvbgsScalars._fields_}

    def _need_init(self):
        if self._shape is None:
            raise LvException(L.NOT_INITIALIZED, "algo must be initialized first")
        return self._shape


class BackgroundSubtractorPAWCS:
    """PAWCS on the GPU, single- and three-channel frames (the lv::CUDA specialisation the reference leaves missing);
    BackgroundSubtractorPAWCS.hpp:47-51 for the constructor parameters."""

    def __init__(self, nDescDistThresholdOffset=2, nMinColorDistThreshold=20, nMaxNbWords=50,
                 nSamplesForMovingAvgs=100, fRelLBSPThreshold=0.333, seed=0, device_id=0, nLBSPThresholdOffset=0,
                 nDefaultMedianBlurKernelSize=9):
        lib = L.lib()
        p = L.LvbgsParams()
        _check(lib.lvbgs_default_params(L.ALGO_PAWCS, C.byref(p)))
        p.desc_dist_threshold_offset = nDescDistThresholdOffset
        p.min_color_dist_threshold = nMinColorDistThreshold
        p.bg_samples = nMaxNbWords
        p.samples_for_moving_avgs = nSamplesForMovingAvgs
        p.rel_lbsp_threshold = fRelLBSPThreshold
        p.lbsp_threshold_offset = nLBSPThresholdOffset
        p.default_median_blur_kernel_size = nDefaultMedianBlurKernelSize
        p.seed = seed
        p.device_id = device_id
        self.params = p
        h = C.c_void_p()
        _check(lib.lvbgs_create(L.ALGO_PAWCS, C.byref(p), C.byref(h)))
        self._h = h
        self._shape = None

    def close(self):
        if self._h:
            L.lib().lvbgs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    initialize = BackgroundSubtractorSuBSENSE.initialize
    apply = BackgroundSubtractorSuBSENSE.apply
    getBackgroundImage = BackgroundSubtractorSuBSENSE.getBackgroundImage
    getBackgroundDescriptorsImage = BackgroundSubtractorSuBSENSE.getBackgroundDescriptorsImage
    setAutomaticModelReset = BackgroundSubtractorSuBSENSE.setAutomaticModelReset
    getDefaultLearningRate = BackgroundSubtractorSuBSENSE.getDefaultLearningRate
    getROICopy = BackgroundSubtractorSuBSENSE.getROICopy
    validateROI = BackgroundSubtractorSuBSENSE.validateROI
    setROI = BackgroundSubtractorSuBSENSE.setROI
    isParallel = BackgroundSubtractorSuBSENSE.isParallel
    getParallelAlgoType = BackgroundSubtractorSuBSENSE.getParallelAlgoType
    _need_init = BackgroundSubtractorSuBSENSE._need_init

    spill = BackgroundSubtractorSuBSENSE.spill
    restore = BackgroundSubtractorSuBSENSE.restore

    def state_bytes(self):
        H, W, Cc = self._need_init()
        return L.lib().lvbgs_state_bytes(L.ALGO_PAWCS, W, H, Cc, self.params.bg_samples)

    def refreshModel(self, nBaseOccCount, fOccDecrFrac, bForceFGUpdate=False):
        _check(L.lib().lvbgs_pawcs_refresh_model(self._h, int(nBaseOccCount), float(fOccDecrFrac),
                                                 1 if bForceFGUpdate else 0), self._h)

    def state_map(self, name):
        """Raw bytes of one model array (include/lvbgs.h, LVBGS_PAWCS_MAP_*; the oracle's layouts)."""
        self._need_init()
        which = L.PAWCS_MAP_NAMES.index(name)
        n = L.lib().lvbgs_pawcs_debug_export_bytes(self._h, which)
        out = np.empty(n, np.uint8)
        _check(L.lib().lvbgs_pawcs_debug_export(self._h, which, out.ctypes.data_as(C.c_void_p), n), self._h)
        return out

    def scalars(self):
        s = L.PawcsScalars()
        _check(L.lib().lvbgs_pawcs_get_scalars(self._h, C.byref(s)), self._h)
        return {f: getattr(s, f) for f, _ in L.PawcsScalars._fields_}


class BackgroundSubtractorLOBSTER:
    """LOBSTER on the GPU, single- and three-channel frames (the non-parallel path of
    BackgroundSubtractorLOBSTER, modules/video/src/BackgroundSubtractorLOBSTER.cpp:410-620);
    BackgroundSubtractorLOBSTER.hpp:50-55 for the constructor parameters and their defaults. apply()'s
    learning rate is LOBSTER's dLearningRate (positive; BGSLOBSTER_DEFAULT_LEARNING_RATE = 16)."""

    def __init__(self, nDescDistThreshold=4, nColorDistThreshold=30, nBGSamples=35, nRequiredBGSamples=2,
                 nLBSPThresholdOffset=0, fRelLBSPThreshold=0.333, seed=0, device_id=0,
                 nDefaultMedianBlurKernelSize=9):
        lib = L.lib()
        p = L.LvbgsParams()
        _check(lib.lvbgs_default_params(L.ALGO_LOBSTER, C.byref(p)))
        p.desc_dist_threshold_offset = nDescDistThreshold
        p.min_color_dist_threshold = nColorDistThreshold
        p.bg_samples = nBGSamples
        p.required_bg_samples = nRequiredBGSamples
        p.rel_lbsp_threshold = fRelLBSPThreshold
        p.lbsp_threshold_offset = nLBSPThresholdOffset
        p.default_median_blur_kernel_size = nDefaultMedianBlurKernelSize
        p.seed = seed
        p.device_id = device_id
        self.params = p
        h = C.c_void_p()
        _check(lib.lvbgs_create(L.ALGO_LOBSTER, C.byref(p), C.byref(h)))
        self._h = h
        self._shape = None

    def close(self):
        if self._h:
            L.lib().lvbgs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    initialize = BackgroundSubtractorSuBSENSE.initialize
    getBackgroundImage = BackgroundSubtractorSuBSENSE.getBackgroundImage
    getBackgroundDescriptorsImage = BackgroundSubtractorSuBSENSE.getBackgroundDescriptorsImage
    refreshModel = BackgroundSubtractorSuBSENSE.refreshModel
    setAutomaticModelReset = BackgroundSubtractorSuBSENSE.setAutomaticModelReset
    getDefaultLearningRate = BackgroundSubtractorSuBSENSE.getDefaultLearningRate
    getROICopy = BackgroundSubtractorSuBSENSE.getROICopy
    validateROI = BackgroundSubtractorSuBSENSE.validateROI
    setROI = BackgroundSubtractorSuBSENSE.setROI
    isParallel = BackgroundSubtractorSuBSENSE.isParallel
    getParallelAlgoType = BackgroundSubtractorSuBSENSE.getParallelAlgoType
    state_map = BackgroundSubtractorSuBSENSE.state_map
    scalars = BackgroundSubtractorSuBSENSE.scalars
    _need_init = BackgroundSubtractorSuBSENSE._need_init

    def apply(self, image, fgmask=None, learningRate=16.0, stream=None):
        """BackgroundSubtractorLOBSTER::apply(image, fgmask, dLearningRate=16) (:459-581)"""
        return BackgroundSubtractorSuBSENSE.apply(self, image, fgmask, learningRate, stream)


class BackgroundSubtractorViBe:
    """ViBe on the GPU: BackgroundSubtractorViBe_1ch on single-channel frames and _3ch on three-channel
    frames (modules/video/src/BackgroundSubtractorViBe.cpp, BackgroundSubtractorViBe.hpp:54-112 for the
    interface and defaults). initialize() takes no ROI; apply()'s learning rate must be positive."""

    def __init__(self, nColorDistThreshold=20, nBGSamples=20, nRequiredBGSamples=2, seed=0, device_id=0):
        lib = L.lib()
        p = L.LvbgsParams()
        _check(lib.lvbgs_default_params(L.ALGO_VIBE, C.byref(p)))
        p.min_color_dist_threshold = nColorDistThreshold
        p.bg_samples = nBGSamples
        p.required_bg_samples = nRequiredBGSamples
        p.seed = seed
        p.device_id = device_id
        self.params = p
        h = C.c_void_p()
        _check(lib.lvbgs_create(L.ALGO_VIBE, C.byref(p), C.byref(h)))
        self._h = h
        self._shape = None

    def close(self):
        if self._h:
            L.lib().lvbgs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    getBackgroundImage = BackgroundSubtractorSuBSENSE.getBackgroundImage
    getDefaultLearningRate = BackgroundSubtractorSuBSENSE.getDefaultLearningRate
    state_map = BackgroundSubtractorSuBSENSE.state_map
    scalars = BackgroundSubtractorSuBSENSE.scalars
    _need_init = BackgroundSubtractorSuBSENSE._need_init

    def initialize(self, oInitImg):
        """initialize(oInitImg) (BackgroundSubtractorViBe.cpp:57-75 / :112-134)"""
        BackgroundSubtractorSuBSENSE.initialize(self, oInitImg, None)

    def apply(self, image, fgmask=None, learningRate=16.0, stream=None):
        """apply(image, fgmask, learningRate=16) (:77-103 / :136-191)"""
        return BackgroundSubtractorSuBSENSE.apply(self, image, fgmask, learningRate, stream)


class BackgroundSubtractorPBAS:
    """PBAS on the GPU: BackgroundSubtractorPBAS_1ch on single-channel frames and _3ch on three-channel
    frames (modules/video/src/BackgroundSubtractorPBAS.cpp, BackgroundSubtractorPBAS.hpp:48-57 and :81-93
    for the interface and defaults). initialize() takes no ROI; apply()'s learningRateOverride replaces
    the per-pixel update rate T(x) when positive (default -1: no override). Maps: SAMPLE_COLOR,
    SAMPLE_GRAD, R, T, DMIN_LT (the D map), GRAD (the last frame's gradient image), MEAN_GRAD."""

    def __init__(self, nInitColorDistThreshold=30, fInitUpdateRate=16.0, nBGSamples=35, nRequiredBGSamples=2,
                 seed=0, device_id=0):
        lib = L.lib()
        p = L.LvbgsParams()
        _check(lib.lvbgs_default_params(L.ALGO_PBAS, C.byref(p)))
        p.min_color_dist_threshold = nInitColorDistThreshold
        p.update_rate = fInitUpdateRate
        p.bg_samples = nBGSamples
        p.required_bg_samples = nRequiredBGSamples
        p.seed = seed
        p.device_id = device_id
        self.params = p
        h = C.c_void_p()
        _check(lib.lvbgs_create(L.ALGO_PBAS, C.byref(p), C.byref(h)))
        self._h = h
        self._shape = None

    close = BackgroundSubtractorViBe.close
    __del__ = BackgroundSubtractorViBe.__del__
    handle = BackgroundSubtractorViBe.handle
    getBackgroundImage = BackgroundSubtractorSuBSENSE.getBackgroundImage
    getDefaultLearningRate = BackgroundSubtractorSuBSENSE.getDefaultLearningRate
    state_map = BackgroundSubtractorSuBSENSE.state_map
    scalars = BackgroundSubtractorSuBSENSE.scalars
    _need_init = BackgroundSubtractorSuBSENSE._need_init

    def initialize(self, oInitImg):
        """initialize(oInitImg) (BackgroundSubtractorPBAS.cpp:61-109 / :287-324)"""
        BackgroundSubtractorSuBSENSE.initialize(self, oInitImg, None)

    def apply(self, image, fgmask=None, learningRateOverride=-1.0, stream=None):
        """apply(image, fgmask, learningRateOverride=-1) (:111-281 / :326-496)"""
        return BackgroundSubtractorSuBSENSE.apply(self, image, fgmask, learningRateOverride, stream)


def map_view(name, raw, W, H, Cc, N):
    """Interprets raw map bytes (reference layout) as a typed numpy array."""
    if name in ("R", "V", "T", "DLAST", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST"):
        return raw.view(np.float32).reshape(H, W)
    if name in ("UNSTABLE", "BLINKS", "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL_INV", "LAST_RAW_BLINK", "ROI"):
        return raw.reshape(H, W)
    if name == "LAST_COLOR":
        return raw.reshape(H, W, Cc)
    if name == "LAST_DESC":
        return raw.view(np.uint16).reshape(H, W, Cc)
    if name in ("SAMPLE_COLOR", "SAMPLE_GRAD"):
        return raw.reshape(N, H, W, Cc)
    if name == "GRAD":
        return raw.reshape(H, W, Cc)
    if name == "MEAN_GRAD":
        return raw.view(np.float32).reshape(1)
    if name == "SAMPLE_DESC":
        return raw.view(np.uint16).reshape(N, H, W, Cc)
    if name in ("DS_LT", "DS_ST"):
        return raw.view(np.float32).reshape(H // 8, W // 8, Cc)
    if name == "LUT":
        return raw.reshape(256)
    raise KeyError(name)


def batch_apply(subtractors, images, masks=None, learning_rates=None, wait=True):
    """One frame of each stream in one call (lvbgs_batch_apply): the SuBSENSE streams in one batched
    frame step, the PAWCS streams' frame steps in flight together on their own CUDA streams."""
    n = len(subtractors)
    if masks is None:
        masks = [np.empty(s._need_init()[:2], np.uint8) for s in subtractors]
    if learning_rates is None:
        learning_rates = [0.0] * n
    hs = (C.c_void_p * n)(*[s.handle for s in subtractors])
    fr = (L.LvbgsFrame * n)()
    keep = []
    for i in range(n):
        ip, k1 = _ptr(images[i])
        mp, k2 = _ptr(masks[i])
        if isinstance(masks[i], np.ndarray) and k2 is not masks[i]:
            raise LvException(L.BAD_ARG, "masks must be C-contiguous uint8 arrays")
        keep += [k1, k2]
        fr[i].image = ip
        fr[i].stride = 0
        fr[i].fgmask = mp
        fr[i].learning_rate = float(learning_rates[i])
    lib = L.lib()
    _check(lib.lvbgs_batch_apply(hs, fr, n, None), subtractors[0].handle)
    if wait:
        _check(lib.lvbgs_batch_wait(hs, n, None), subtractors[0].handle)
    return masks


def lbsp_compute2(image, abs_threshold=None, rel_threshold=0.333, offset=0, device_id=0):
    """Dense LBSP descriptors on the device (LBSP::compute2, modules/features2d/src/LBSP.cpp:102-152)."""
    H, W, Cc = _shape(image)
    img = np.ascontiguousarray(image, dtype=np.uint8)
    out = np.zeros((H, W, Cc) if Cc > 1 else (H, W), np.uint16)
    thr = -1 if abs_threshold is None else int(abs_threshold)
    _check(L.lib().lvbgs_lbsp_compute2(img.ctypes.data_as(C.c_void_p), W, H, Cc, thr, float(rel_threshold),
                                       int(offset), out.ctypes.data_as(C.c_void_p), device_id))
    return out
