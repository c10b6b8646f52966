"""CPU tests of the C-ABI library: it loads, exports every declared entry point, and its host-only
parts (parameters, sizes, synthetic generator) behave; no compute call needs a GPU here."""
import ctypes as C
import glob
import os
import re

import numpy as np

from litiv_gb300 import _lib as L

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = set()
    for path in glob.glob(os.path.join(INCLUDE, "*.h")):
        src = open(path).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:lvbgs|lvsynth|lvserve)_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(product_lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in sorted(names) if not hasattr(product_lib, n)]
    assert not missing, missing
    assert set(L.SIGNATURES) >= names


def test_default_params_match_reference(product_lib):
    p = L.LvbgsParams()
    assert product_lib.lvbgs_default_params(L.ALGO_SUBSENSE, C.byref(p)) == L.OK
    # BackgroundSubtractorSuBSENSE.hpp:22-31, BackgroundSubtractorLBSP.hpp:23-28
    assert (p.desc_dist_threshold_offset, p.min_color_dist_threshold, p.bg_samples, p.required_bg_samples,
            p.samples_for_moving_avgs, p.lbsp_threshold_offset, p.default_median_blur_kernel_size) == (
                3, 30, 50, 2, 100, 0, 9)
    assert abs(p.rel_lbsp_threshold - 0.333) < 1e-7
    # BackgroundSubtractorPAWCS.hpp:22-29: offset 2, colour 20, 50 words, 100 frames
    assert product_lib.lvbgs_default_params(L.ALGO_PAWCS, C.byref(p)) == L.OK
    assert (p.desc_dist_threshold_offset, p.min_color_dist_threshold, p.bg_samples, p.samples_for_moving_avgs,
            p.default_median_blur_kernel_size) == (2, 20, 50, 100, 9)
    # BackgroundSubtractorLOBSTER.hpp:22-31: descriptor 4, colour 30, 35 samples, 2 required
    assert product_lib.lvbgs_default_params(L.ALGO_LOBSTER, C.byref(p)) == L.OK
    assert (p.desc_dist_threshold_offset, p.min_color_dist_threshold, p.bg_samples, p.required_bg_samples,
            p.lbsp_threshold_offset, p.default_median_blur_kernel_size) == (4, 30, 35, 2, 0, 9)
    assert abs(p.rel_lbsp_threshold - 0.333) < 1e-7
    # BackgroundSubtractorViBe.hpp:39-46: colour 20, 20 samples, 2 required
    assert product_lib.lvbgs_default_params(L.ALGO_VIBE, C.byref(p)) == L.OK
    assert (p.min_color_dist_threshold, p.bg_samples, p.required_bg_samples) == (20, 20, 2)
    # BackgroundSubtractorPBAS.hpp:48-55: colour 30, update rate 16, 35 samples, 2 required
    assert product_lib.lvbgs_default_params(L.ALGO_PBAS, C.byref(p)) == L.OK
    assert (p.min_color_dist_threshold, p.update_rate, p.bg_samples, p.required_bg_samples) == (30, 16.0, 35, 2)
    assert product_lib.lvbgs_default_params(7, C.byref(p)) == L.BAD_ARG


def test_create_rejects_bad_parameters(product_lib):
    p = L.LvbgsParams()
    product_lib.lvbgs_default_params(L.ALGO_SUBSENSE, C.byref(p))
    p.required_bg_samples = 51
    h = C.c_void_p()
    assert product_lib.lvbgs_create(L.ALGO_SUBSENSE, C.byref(p), C.byref(h)) == L.BAD_ARG
    assert b"more sample matches" in product_lib.lvbgs_last_error(None)
    product_lib.lvbgs_default_params(L.ALGO_SUBSENSE, C.byref(p))
    p.min_color_dist_threshold = 0
    p.desc_dist_threshold_offset = 0
    assert product_lib.lvbgs_create(L.ALGO_SUBSENSE, C.byref(p), C.byref(h)) == L.BAD_ARG
    product_lib.lvbgs_default_params(L.ALGO_SUBSENSE, C.byref(p))
    p.bg_samples = 65
    assert product_lib.lvbgs_create(L.ALGO_SUBSENSE, C.byref(p), C.byref(h)) == L.UNSUPPORTED
    # PBAS's update rate must be in (0, 255] (BackgroundSubtractorPBAS.cpp:32)
    for rate in (0.0, -1.0, 256.0, float("nan")):
        product_lib.lvbgs_default_params(L.ALGO_PBAS, C.byref(p))
        p.update_rate = rate
        assert product_lib.lvbgs_create(L.ALGO_PBAS, C.byref(p), C.byref(h)) == L.BAD_ARG


def test_null_handle_calls_fail_cleanly(product_lib):
    assert product_lib.lvbgs_apply(None, None, 0, None, 0.0, None) == L.BAD_ARG
    assert product_lib.lvbgs_initialize(None, None, 1, 1, 1, 0, None) == L.BAD_ARG
    assert product_lib.lvbgs_destroy(None) == L.OK
    assert product_lib.lvbgs_batch_apply(None, None, 0, None) == L.BAD_ARG


def test_state_bytes_accounts_for_the_model(product_lib):
    b3 = product_lib.lvbgs_state_bytes(L.ALGO_SUBSENSE, 320, 240, 3, 50)
    b1 = product_lib.lvbgs_state_bytes(L.ALGO_SUBSENSE, 320, 240, 1, 50)
    npx = 320 * 240
    # 50 samples x 3c bytes + 10 double-buffered float maps + the rest
    assert b3 >= npx * (50 * 9 + 80) and b1 >= npx * (50 * 3 + 80)
    assert b3 > b1 > 0
    assert product_lib.lvbgs_state_bytes(L.ALGO_SUBSENSE, 0, 240, 3, 50) == 0


def test_pawcs_state_bytes_for_one_and_three_channels(product_lib):
    # 640x480: 25 local words (one channel) or 50 (three), each double-buffered with colour,
    # descriptor and three 32-bit counters; four-channel frames are not a PAWCS input
    npx = 640 * 480
    b1 = product_lib.lvbgs_state_bytes(L.ALGO_PAWCS, 640, 480, 1, 0)
    b3 = product_lib.lvbgs_state_bytes(L.ALGO_PAWCS, 640, 480, 3, 0)
    assert b1 >= npx * 2 * 25 * (1 + 2 + 12)
    assert b3 >= npx * 2 * 50 * (3 + 6 + 12)
    assert product_lib.lvbgs_device_bytes(L.ALGO_PAWCS, 640, 480, 3, 0) > b3
    assert product_lib.lvbgs_state_bytes(L.ALGO_PAWCS, 640, 480, 4, 0) == 0


def test_synthetic_presets_and_determinism(product_lib):
    from litiv_gb300 import SyntheticStream
    s = SyntheticStream(0, seed=1)
    f0, g0 = s.render(5, with_gt=True)
    f1, g1 = s.render(5, with_gt=True)
    np.testing.assert_array_equal(f0, f1)
    assert f0.shape == (240, 320, 3) and 0.005 < (g0 > 0).mean() < 0.3
    assert 15 < f0.std() < 60
    assert not np.array_equal(f0, SyntheticStream(0, seed=2).render(5))
    sizes, gray = {}, 0
    for i in range(64):
        c = SyntheticStream(3, index=i, seed=1).cfg
        sizes[(c.width, c.height)] = sizes.get((c.width, c.height), 0) + 1
        gray += c.channels == 1
        assert 2000 <= c.noise_sigma_milli <= 6000 and 2 <= c.n_shapes <= 10
    assert sizes == {(320, 240): 16, (640, 480): 24, (1280, 720): 16, (1920, 1080): 8} and gray == 16
