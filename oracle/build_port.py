"""Builds the oracle port (oracle/pppm_port.cc) into oracle/_build/libpppm_port.so.

Test infrastructure: compiled on every machine (the GPU machine included) by
__graft_entry__.build(), because tests and bench.py's CPU-baseline leg load
it there. -ffp-contract=off keeps double arithmetic rounded step by step,
as the reference's x86-64 build does (it has no FMA without -march).
"""
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "pppm_port.cc"
OUT = HERE / "_build" / "libpppm_port.so"


def build() -> pathlib.Path:
    OUT.parent.mkdir(exist_ok=True)
    deps = [SRC, HERE.parent / "include" / "pppm_c.h"]
    if OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", str(SRC), "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle port build failed:\n" + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build())
