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


def test_noalloc_pointer_rule(tmp_path):
    """pppm_knn_noalloc stages nothing, so it takes only memory its kernels
    read in place on the current device: that device's own memory or managed
    memory. Another GPU's memory (an illegal address without peer access),
    host and unregistered memory are refused. The rule is checked here on
    the host with the memory types and device ordinals that
    cudaPointerGetAttributes reports, so no GPU ever sees a foreign pointer."""
    import shutil
    import subprocess

    if shutil.which("g++") is None:
        pytest.skip("no host compiler")
    src = tmp_path / "rule.cc"
    src.write_text(
        '#include "noalloc_check.h"\n#include <cstdio>\nusing namespace pppm;\n'
        "int main() {\n"
        "  int bad = 0;\n"
        "  bad += !naPointerUsable(kNaDevice, 0, 0);\n"
        "  bad += !naPointerUsable(kNaDevice, 3, 3);\n"
        "  bad += naPointerUsable(kNaDevice, 1, 0);\n"
        "  bad += naPointerUsable(kNaDevice, 0, 1);\n"
        "  bad += !naPointerUsable(kNaManaged, 0, 1);\n"
        "  bad += !naPointerUsable(kNaManaged, -2, 0);\n"
        "  bad += naPointerUsable(kNaHost, 0, 0);\n"
        "  bad += naPointerUsable(kNaUnregistered, 0, 0);\n"
        '  std::printf("%d\\n", bad);\n  return bad;\n}\n')
    exe = tmp_path / "rule"
    subprocess.run(["g++", "-std=c++17", "-I", str(P.HERE / "csrc"), str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
