"""GPU tests of the frame precacher (lvbgs_precacher_*, lv::DataPrecacher of
modules/datasets/src/utils.cpp:302-470): packets come back byte for byte in and out of order, with and
without precaching, the stream ends at the first empty packet, loader failures are reported, and masks
computed from precached device frames equal masks from host frames."""
import ctypes as C

import numpy as np
import pytest

from litiv_gb300 import BackgroundSubtractorSuBSENSE, DataPrecacher, LvException, SyntheticStream
from litiv_gb300 import _lib as L

pytestmark = pytest.mark.gpu

_D2H = 2  # cudaMemcpyDeviceToHost


def device_bytes(pkt):
    out = np.empty(pkt.nbytes, np.uint8)
    cudart = L.lib()  # the library's CUDA runtime, found through its dependencies
    cudart.cudaDeviceSynchronize()
    assert cudart.cudaMemcpy(out.ctypes.data_as(C.c_void_p), C.c_void_p(pkt.data_ptr()), C.c_size_t(pkt.nbytes),
                             _D2H) == 0
    return out


def packets(n, nbytes=200_003, seed=0):
    return np.random.default_rng(seed).integers(0, 256, size=(n, nbytes), dtype=np.uint8)


@pytest.mark.parametrize("precache", [False, True])
def test_sequential_and_out_of_order_requests(precache):
    arr = packets(40)
    pc = DataPrecacher(arr)
    if precache:
        assert pc.startAsyncPrecaching(6 * arr[0].nbytes)
    order = list(range(0, 25)) + [30, 31, 32, 3, 4, 5, 39, 12, 12, 13]
    for i in order:
        pkt = pc.getPacket(i)
        assert pkt.nbytes == arr[0].nbytes
        assert np.array_equal(pkt.host, arr[i]), i
        assert np.array_equal(device_bytes(pkt), arr[i]), i
        assert pc.getLastReqIdx() == i
    # past the end of the stream: an empty packet
    assert pc.getPacket(40) is None
    assert pc.getPacket(41) is None
    assert np.array_equal(device_bytes(pc.getPacket(7)), arr[7])
    pc.stopAsyncPrecaching()
    assert not pc.isActive()
    pc.close()


def test_python_loader_end_and_errors():
    arr = packets(12, 50_000, seed=1)

    def load(i):
        if i == 9:
            raise RuntimeError("broken packet")
        return arr[i] if i < 12 else None

    pc = DataPrecacher(load, max_packet_bytes=arr[0].nbytes)
    pc.startAsyncPrecaching(4 * arr[0].nbytes)
    for i in range(9):
        assert np.array_equal(device_bytes(pc.getPacket(i)), arr[i])
    with pytest.raises(LvException) as ei:
        pc.getPacket(9)
    assert ei.value.status == L.BAD_ARG
    with pytest.raises(LvException):
        pc.stopAsyncPrecaching()
    # without precaching, packets after the failing one still load on demand
    assert np.array_equal(device_bytes(pc.getPacket(10)), arr[10])
    assert pc.getPacket(12) is None
    pc.close()


def test_long_run_through_a_small_ring():
    arr = packets(150, 70_001, seed=2)
    pc = DataPrecacher(arr)
    pc.startAsyncPrecaching(2 * arr[0].nbytes)  # the minimum ring: one packet handed, one loading
    for i in range(150):
        assert np.array_equal(device_bytes(pc.getPacket(i)), arr[i]), i
    pc.close()


def test_masks_from_precached_frames_equal_masks_from_host_frames():
    import torch
    s = SyntheticStream(0, 0, 3)
    frames = np.stack([s.render(t) for t in range(50)])
    ref = BackgroundSubtractorSuBSENSE(seed=9)
    ref.initialize(frames[0])
    want = [ref.apply(f) for f in frames[1:]]
    pc = DataPrecacher(frames)
    pc.startAsyncPrecaching(8 * frames[0].nbytes)
    m = BackgroundSubtractorSuBSENSE(seed=9)
    stream = torch.cuda.Stream()
    first = pc.getPacket(0, stream)
    m.initialize(first.host.copy())
    for t in range(1, 50):
        pkt = pc.getPacket(t, stream)
        assert pkt.shape == frames[t].shape
        got = m.apply(pkt, stream=stream)
        assert np.array_equal(got, want[t - 1]), t
    pc.close()


def test_argument_checks():
    h = C.c_void_p()
    assert L.lib().lvbgs_precacher_create(None, None, 100, 0, C.byref(h)) == L.BAD_ARG
    arr = packets(3, 1000)
    with pytest.raises(LvException):
        DataPrecacher(arr, max_packet_bytes=10).getPacket(0)  # the packets do not fit the capacity


def test_packets_in_pinned_host_memory_are_uploaded_in_place():
    import torch
    arr = packets(30, 123_456, seed=3)
    pinned = torch.from_numpy(arr).pin_memory()
    h = C.c_void_p()
    assert L.lib().lvbgs_precacher_create_host(C.c_void_p(pinned.data_ptr()), arr.shape[1], arr.shape[0], 0,
                                               C.byref(h)) == L.OK
    dp, hp, sz = C.c_void_p(), C.c_void_p(), C.c_size_t()

    class Pkt:
        def __init__(self):
            self.nbytes = sz.value

        def data_ptr(self):
            return dp.value

    for start in (False, True):
        if start:
            assert L.lib().lvbgs_precacher_start(h, 3 * arr.shape[1]) == L.OK
        for i in list(range(12)) + [20, 21, 5, 29]:
            assert L.lib().lvbgs_precacher_get(h, i, None, C.byref(dp), C.byref(hp), C.byref(sz)) == L.OK
            assert sz.value == arr.shape[1]
            # the host copy is the caller's own memory
            assert hp.value == pinned.data_ptr() + i * arr.shape[1]
            assert np.array_equal(device_bytes(Pkt()), arr[i]), (start, i)
        assert L.lib().lvbgs_precacher_get(h, 30, None, C.byref(dp), C.byref(hp), C.byref(sz)) == L.OK
        assert sz.value == 0
    assert L.lib().lvbgs_precacher_destroy(h) == L.OK
