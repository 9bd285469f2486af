"""The host QBVH construction builds large subtrees as parallel tasks and
appends them in child order; its layout must equal the serial one (the
tree, the leaf slot order, the root and depth) whatever the thread count."""
import os
import pathlib
import subprocess

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "tatsy-pppm_gb300" / "csrc"


def test_parallel_qbvh_build_equals_serial(tmp_path):
    exe = tmp_path / "qbvh_build_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", f"-I{CSRC}",
                    str(ROOT / "tests" / "qbvh_build_check.cc"), str(CSRC / "host_build.cc"), "-o", str(exe)],
                   check=True, capture_output=True, timeout=300)
    outs = {}
    for threads in (1, 2, 5):
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        outs[threads] = subprocess.run([str(exe)], check=True, capture_output=True, text=True, env=env,
                                       timeout=300).stdout
    assert outs[1].count("\n") == 8 and "error" not in outs[1]
    assert outs[1] == outs[2] == outs[5]
