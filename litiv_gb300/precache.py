"""Host-side mirror of lv::DataPrecacher (modules/datasets/include/litiv/datasets/utils.hpp:456-478) for a
GPU consumer, bound to the C-ABI (lvbgs_precacher_* in include/lvbgs.h).

``DataPrecacher(loader, max_packet_bytes)`` takes the reference's loader callback (packet index -> packet,
an empty or None packet ending the stream) or an array of packets already in host memory (loaded by the
library's own copy loader, without the interpreter). ``getPacket(idx)`` returns a ``DevicePacket``: its
``data_ptr()`` is the device copy (so it can be passed wherever a CUDA tensor is accepted, e.g.
``BackgroundSubtractorSuBSENSE.apply``) and ``host`` the pinned host copy; it stays valid until the next
``getPacket`` with another index.
"""
import ctypes as C

import numpy as np

from . import _lib as L
from .bgs import LvException, _check


class DevicePacket:
    """A packet handed out by the precacher: device pointer, pinned host view and packet shape."""

    def __init__(self, dev_ptr, host_ptr, size, shape):
        self._dev = dev_ptr
        self.nbytes = size
        self.shape = tuple(shape) if shape is not None else (size,)
        self.host = np.ctypeslib.as_array((C.c_uint8 * size).from_address(host_ptr)).reshape(self.shape)

    def data_ptr(self):
        return self._dev


class DataPrecacher:
    def __init__(self, loader, max_packet_bytes=None, shape=None, device_id=0):
        self._shape = shape
        self._keep = []
        lib = L.lib()
        if isinstance(loader, np.ndarray):
            packets = np.ascontiguousarray(loader, dtype=np.uint8)
            self._keep.append(packets)
            self._packets = L.HostPackets(packets.ctypes.data, packets[0].nbytes if len(packets) else 0, len(packets))
            fn = C.cast(lib.lvbgs_precache_copy_loader, C.c_void_p)
            user = C.cast(C.pointer(self._packets), C.c_void_p)
            max_packet_bytes = max_packet_bytes or max(1, self._packets.packet_bytes)
            if self._shape is None and len(packets):
                self._shape = packets.shape[1:]
        else:
            if not callable(loader):
                raise LvException(L.BAD_ARG, "invalid data precacher callback")
            if not max_packet_bytes:
                raise LvException(L.BAD_ARG, "a loader callback needs max_packet_bytes")

            def call(_user, idx, dst, cap):
                try:
                    pkt = loader(int(idx))
                except Exception:
                    return cap + 1  # reported as a loader error
                if pkt is None:
                    return 0
                pkt = np.ascontiguousarray(pkt, dtype=np.uint8)
                if pkt.nbytes > cap:
                    return cap + 1
                C.memmove(dst, pkt.ctypes.data, pkt.nbytes)
                return pkt.nbytes

            self._cb = L.PACKET_LOADER(call)
            fn = C.cast(self._cb, C.c_void_p)
            user = None
        self._h = C.c_void_p()
        _check(lib.lvbgs_precacher_create(fn, user, int(max_packet_bytes), int(device_id), C.byref(self._h)))

    def close(self):
        if self._h:
            L.lib().lvbgs_precacher_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def startAsyncPrecaching(self, nSuggestedBufferSize):
        _check(L.lib().lvbgs_precacher_start(self._h, int(nSuggestedBufferSize)))
        return self.isActive()

    def stopAsyncPrecaching(self):
        _check(L.lib().lvbgs_precacher_stop(self._h))

    def isActive(self):
        return bool(L.lib().lvbgs_precacher_is_active(self._h))

    def getLastReqIdx(self):
        v = L.lib().lvbgs_precacher_last_index(self._h)
        return None if v == (1 << 64) - 1 else v

    def getPacket(self, idx, stream=None):
        """The packet `idx` (None past the end of the stream); `stream` (a cudaStream_t as int, or a
        torch.cuda.Stream) is made to wait for its upload (default: the legacy default stream)."""
        if stream is not None and hasattr(stream, "cuda_stream"):
            stream = stream.cuda_stream
        dev, host, size = C.c_void_p(), C.c_void_p(), C.c_size_t()
        _check(L.lib().lvbgs_precacher_get(self._h, int(idx), C.c_void_p(stream) if stream else None, C.byref(dev),
                                           C.byref(host), C.byref(size)))
        if size.value == 0:
            return None
        shape = self._shape if self._shape is not None and int(np.prod(self._shape)) == size.value else None
        return DevicePacket(dev.value, host.value, size.value, shape)
