"""Generates the LBSP known-answer fixtures from the reference's own test data.

The reference pins its LBSP descriptor with ``lbsp.regression_compute``
(modules/features2d/test/lbsp.cpp:22-46): ``LBSP(20)`` (absolute threshold 20)
is run through ``compute2`` on a 65x65 BGR crop of
``samples/data/multispectral_stereo_ex/img2.png`` whose top-left corner is
(371-2-30, 371-2-30) = (339, 339), and the result is compared with
``modules/features2d/test/data/test_lbsp.bin`` on the inner 61x61 zone.

This script (run once, in a container where the reference tree is mounted)
decodes the PNG with zlib (8-bit RGB, no interlace; OpenCV's imread gives BGR
order, so channels are reversed), takes the same crop, and parses the
``lv::write`` binary archive (modules/utils/src/opencv.cpp:514-531: int32 type,
uint64 elemSize, uint64 count, int32 dims, int32 sizes[dims], raw data).
It writes two small .npy fixtures next to itself:

* ``lbsp_input_65x65_bgr.npy``  uint8 [65,65,3]
* ``lbsp_abs20_65x65_u16c3.npy`` uint16 [65,65,3]
"""
import os
import struct
import sys
import zlib

import numpy as np

REF_ROOT = os.environ.get("LITIV_REFERENCE_ROOT", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    if pb <= pc:
        return b
    return c


def decode_png_rgb8(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos, idat, hdr = 8, bytearray(), None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        ctype = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if ctype == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif ctype == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, color, _, _, interlace = hdr
    assert depth == 8 and color == 2 and interlace == 0, hdr
    raw = zlib.decompress(bytes(idat))
    bpp, stride = 3, w * 3
    out = np.zeros((h, stride), np.uint8)
    prev = [0] * stride
    i = 0
    for y in range(h):
        ftype = raw[i]
        line = list(raw[i + 1:i + 1 + stride])
        i += 1 + stride
        for x in range(stride):
            a = line[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if ftype == 1:
                line[x] = (line[x] + a) & 255
            elif ftype == 2:
                line[x] = (line[x] + b) & 255
            elif ftype == 3:
                line[x] = (line[x] + ((a + b) >> 1)) & 255
            elif ftype == 4:
                line[x] = (line[x] + _paeth(a, b, c)) & 255
            else:
                assert ftype == 0, ftype
        out[y] = line
        prev = line
    return out.reshape(h, w, 3)


def read_lv_archive(path):
    d = open(path, "rb").read()
    dtype, elem, count, dims = struct.unpack("<iQQi", d[:24])
    sizes = struct.unpack("<%di" % dims, d[24:24 + 4 * dims])
    payload = d[24 + 4 * dims:]
    assert len(payload) == elem * count
    assert dtype == 18 and elem == 6  # CV_16UC3
    return np.frombuffer(payload, np.uint16).reshape(*sizes, 3).copy()


def main():
    png = os.path.join(REF_ROOT, "samples/data/multispectral_stereo_ex/img2.png")
    golden = os.path.join(REF_ROOT, "modules/features2d/test/data/test_lbsp.bin")
    rgb = decode_png_rgb8(png)
    bgr = rgb[:, :, ::-1]
    x0 = y0 = 371 - 2 - 30
    crop = np.ascontiguousarray(bgr[y0:y0 + 65, x0:x0 + 65])
    desc = read_lv_archive(golden)
    assert desc.shape == (65, 65, 3)
    np.save(os.path.join(HERE, "lbsp_input_65x65_bgr.npy"), crop)
    np.save(os.path.join(HERE, "lbsp_abs20_65x65_u16c3.npy"), desc)
    print("wrote fixtures", crop.shape, desc.shape)


if __name__ == "__main__":
    sys.exit(main())
