"""PNG encoder of the output stage (host only): a file any PNG reader
decodes to the same pixels (signature, chunk CRCs, zlib stream, rows)."""
import struct
import zlib

import numpy as np
import pytest

import pppm_gb300 as P


@pytest.mark.parametrize("shape", [(1, 1), (7, 13), (64, 100)])
def test_png_decodes_to_the_pixels(shape):
    h, w = shape
    img = np.random.default_rng(h * 1000 + w).integers(0, 256, (h, w, 3), dtype=np.uint8)
    data = P.png_encode(img)
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        chunks.append((typ, body))
        pos += 12 + n
    assert [t for t, _ in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    assert struct.unpack(">IIBBBBB", chunks[0][1]) == (w, h, 8, 2, 0, 0, 0)
    raw = zlib.decompress(chunks[1][1])
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert (rows[:, 0] == 0).all()
    assert np.array_equal(rows[:, 1:].reshape(h, w, 3), img)


def test_png_size_query_and_capacity():
    img = np.zeros((4, 5, 3), np.uint8)
    lib = P.load()
    import ctypes
    n = ctypes.c_int64()
    assert lib.pppm_png_encode(img.ctypes.data, 5, 4, None, 0, ctypes.byref(n)) == P.OK
    small = np.zeros(n.value - 1, np.uint8)
    assert lib.pppm_png_encode(img.ctypes.data, 5, 4, small.ctypes.data, small.size, ctypes.byref(n)) == P.E_CAPACITY
