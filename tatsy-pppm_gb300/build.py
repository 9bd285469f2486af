"""Build recipe for libpppm_gb300.so (sm_103a only).

Every .cu in csrc/ is compiled by nvcc for `-gencode arch=compute_103a,code=sm_103a`
and every .cc by the host compiler, in parallel, then linked into
tatsy-pppm_gb300/libpppm_gb300.so. Objects go to tatsy-pppm_gb300/_build/.
Run directly (`python tatsy-pppm_gb300/build.py`) or through
__graft_entry__.build().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = HERE / "libpppm_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# extra nvcc flags for tuning builds (e.g. -DPPPM_TRACE_MINBLOCKS=4)
EXTRA = os.environ.get("PPPM_NVCC_EXTRA", "").split()


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(src: pathlib.Path, obj: pathlib.Path, deps):
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def build(verbose: bool = False, ptxas_info: bool = False) -> pathlib.Path:
    OUT.mkdir(exist_ok=True)
    # rebuild everything when the extra flags change
    stamp = OUT / "flags.txt"
    flags = " ".join(EXTRA)
    if not stamp.exists() or stamp.read_text() != flags:
        for o in OUT.glob("*.o"):
            o.unlink()
        stamp.write_text(flags)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "pppm_c.h"]
    jobs = []
    objs = []
    nvcc = _nvcc()
    for src in sorted(CSRC.glob("*.cu")):
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        if _stale(src, obj, headers) or ptxas_info:
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "--expt-relaxed-constexpr", *EXTRA, "-c", str(src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in sorted(CSRC.glob("*.cc")):
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        if _stale(src, obj, headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", "-c", str(src), "-o",
                         str(obj)])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", str(LIB), *map(str, objs)])
    demo = HERE / "appmain_gpu"
    src = HERE / "host" / "appmain_gpu.cc"
    if not demo.exists() or demo.stat().st_mtime < max(LIB.stat().st_mtime, src.stat().st_mtime,
                                                       (HERE / "host" / "pppm.hpp").stat().st_mtime):
        _run(["g++", "-std=c++17", "-O2", str(src), "-o", str(demo), f"-L{HERE}", "-lpppm_gb300",
              f"-Wl,-rpath,{HERE}"])
    if verbose or ptxas_info:
        for s in logs:
            if s.strip():
                print(s)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
