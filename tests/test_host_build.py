"""The host QBVH construction builds large subtrees as parallel tasks that
write straight into their places of the serial depth-first layout; its
layout (the tree, the leaf slot order, the root and depth) must equal the
serial one whatever the thread count, and must stay the one the serial
construction gave (hashes below), which the renders' closest-hit parity
with the reference rests on."""
import os
import pathlib
import subprocess

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "tatsy-pppm_gb300" / "csrc"
# size, nodes, layout hash of each seeded soup, from the serial construction
SERIAL_LAYOUT = """\
1 0 cbbb1c7408d12174
3 0 388d457e2a3edef4
4 1 b733e1e4e0207bee
17 5 86592571a93a02fc
1000 277 15e46a047cebec86
16384 5461 ea8b45e6881dffc2
70000 21845 daebe57045676fc3
200000 25237 f3d4736d3b6eff4e
"""


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
    assert outs[1] == SERIAL_LAYOUT
