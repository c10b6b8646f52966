"""GPU test of lvbgs_lbsp_compute2_noalloc, the LBSP entry point that allocates no device memory.

Callers that must not call cudaMalloc/cudaFree -- a real-time capture thread under a
no-allocation rule, or a process held to a fixed GPU memory budget -- use this entry point; it
stages its data in one file-scope device array that the CUDA runtime reserves when the library is
first used on the device. This test calls it through the C-ABI twice in a row (so the second call
runs on an array that still holds the first call's data) and compares each result with
lvbgs_lbsp_compute2, the allocating entry point. Descriptors are integers, so the tolerance is
zero: the outputs must be identical. After the first call, free device memory must not change
across a call. The file sorts last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from litiv_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _free_device_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize(0)
    return torch.cuda.mem_get_info(0)[0]


def test_noalloc_matches_allocating_entry_point_twice_in_a_row():
    lib = L.lib()
    rng = np.random.default_rng(11)
    # (shape, channels, absolute threshold or -1 for the relative threshold 0.333 with offset 2)
    cases = [((480, 640), 1, 20), ((720, 1280, 3), 3, -1), ((1080, 1920, 3), 3, 20)]
    for call in range(2):
        for shape, c, thr in cases:
            img = rng.integers(0, 256, shape, dtype=np.uint8)
            border = rng.integers(0, 65536, shape, dtype=np.uint16)  # the 2-pixel border keeps the caller's data
            ref = border.copy()
            out = border.copy()
            H, W = shape[0], shape[1]
            st = lib.lvbgs_lbsp_compute2(_ptr(img), W, H, c, thr, 0.333, 2, _ptr(ref), 0)
            assert st == L.OK, lib.lvbgs_last_error(None)
            free0 = _free_device_bytes() if call == 1 else None
            st = lib.lvbgs_lbsp_compute2_noalloc(_ptr(img), W, H, c, thr, 0.333, 2, _ptr(out), 0, None)
            assert st == L.OK, lib.lvbgs_last_error(None)
            if call == 1:
                # the array and the kernel were set up by the first call: this one allocates nothing
                assert _free_device_bytes() == free0
            np.testing.assert_array_equal(out, ref)


def test_noalloc_rejects_frames_above_its_fixed_scratch():
    lib = L.lib()
    one = np.zeros(1, np.uint8)
    desc = np.zeros(1, np.uint16)
    # 2048 x 1366 x 3 = 8,392,704 elements > 8,388,608; rejected before any device work
    st = lib.lvbgs_lbsp_compute2_noalloc(_ptr(one), 2048, 1366, 3, 20, 0.333, 0, _ptr(desc), 0, None)
    assert st == L.BAD_SIZE
    assert b"8,388,608" in lib.lvbgs_last_error(None)
