"""The CCD search's path encoding (rigid-ipc_gb300/csrc/search_tree.cuh)
compiled as plain C++ and checked on the CPU against an explicit box stack:
the same boxes in the same order, the same bottom box for work sharing, the
same smallest pending t.lo, exact dyadic bounds and root-finder widths
(tests/search_tree_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "rigid-ipc_gb300", "csrc")


def test_path_encoding_matches_box_stack(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "search_tree_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "search_tree_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok"), out.stdout
    assert int(out.stdout.split()[1]) > 1_000_000
