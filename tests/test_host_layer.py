"""The C++ host layer (reference-named classes over the C ABI) compiles, and
a C++ caller links against the library without CUDA symbols of its own."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

HDR = os.path.join(ROOT, "rigid-ipc_gb300", "host", "rigid_ipc_gb300.hpp")

CALLER = r"""
#include "rigid_ipc_gb300.hpp"
using namespace ipc::rigid::gb300;
double narrow_phase(DistanceBarrierRBProblem& p, const std::vector<double>& x0,
                    const std::vector<double>& x1, std::vector<double>& g, BlockSparse& H)
{
    double toi = p.compute_earliest_toi(x0, x1);
    double e = p.compute_barrier_term(x0, g, H, true, true);
    Candidates c;
    detect_collision_candidates_rigid(p.assembler(), x0, x1, c);
    return toi + e + c.size();
}
"""


def _cuda_include():
    for p in ("/usr/local/cuda/include", "/usr/local/cuda/targets/x86_64-linux/include",
              "/usr/local/cuda/targets/sbsa-linux/include"):
        if os.path.exists(os.path.join(p, "cuda_runtime.h")):
            return p
    return None


def test_host_layer_compiles(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("g++ or CUDA headers not available")
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-I", os.path.dirname(HDR),
                        "-I", inc, str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
