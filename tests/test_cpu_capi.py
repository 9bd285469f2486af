"""CPU-side checks of the C-ABI library (no GPU needed).

The shared object must load and export every function declared in
include/pppm_c.h; host-only entry points run here; entry points that need a
device fail with a status code instead of aborting.
"""
import ctypes

import numpy as np
import pytest

import pppm_gb300 as P


def _lib():
    if not P.LIB_PATH.exists():
        pytest.skip("libpppm_gb300.so not built")
    return P.load()


def test_exports_every_declared_symbol():
    lib = _lib()
    names = P.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(P.SIGNATURES) == set(names), set(P.SIGNATURES) ^ set(names)


def test_hdr_decode_matches_reference_loader(golden):
    _lib()
    g = golden("env")
    rgb = P.hdr_decode(g["hdr_bytes"].tobytes())
    # Image::loadHdr yields doubles that are exact floats (8-bit mantissa * 2^e)
    assert np.array_equal(rgb, g["decoded"].astype(np.float32))


def test_hdr_decode_rejects_corrupt_input(golden):
    _lib()
    g = golden("env")
    data = g["hdr_bytes"].tobytes()
    for bad in (data[:20], b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 4 +X 4\n" + b"\x01" * 8, data[: len(data) // 2]):
        with pytest.raises(P.PppmError):
            P.hdr_decode(bad)


def test_null_and_bad_arguments_return_status():
    lib = _lib()
    assert lib.pppm_destroy(None) == P.E_ARG
    assert lib.pppm_sync(None) == P.E_ARG
    assert lib.pppm_last_error(None) == b"null context"
    h = ctypes.c_void_p()
    r = lib.pppm_create(-1, ctypes.byref(h))
    assert r == P.E_CUDA and not h.value

