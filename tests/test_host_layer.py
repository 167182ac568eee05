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


def _write_vec(f, a, dtype):
    import numpy as np

    a = np.ascontiguousarray(np.asarray(a, dtype=dtype).reshape(-1))
    f.write(np.int64(a.size).tobytes())
    f.write(a.tobytes())


def _read_vec(f, dtype):
    import numpy as np

    n = int(np.frombuffer(f.read(8), np.int64)[0])
    return np.frombuffer(f.read(n * np.dtype(dtype).itemsize), dtype=dtype)


@pytest.mark.gpu
def test_host_layer_runs_and_matches_binding(tmp_path):
    """Build the C++ caller against librigc.so, run one narrow-phase pass
    of the stacked 27-cube contact through the reference-named classes, and
    compare every output with the Python binding's on the same inputs: time
    of impact (rigid and piecewise-linear trajectories), barrier energy,
    gradient, block-sparse Hessian, candidates, minimum distance and the
    intersection check, bit for bit."""
    import numpy as np

    import rigc
    from conftest import contact_poses
    from rigc import scene as S

    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("g++ or CUDA headers not available")
    lib_dir = os.path.join(ROOT, "rigid-ipc_gb300", "_build")
    cuda_lib = os.path.join(os.path.dirname(inc), "lib64")
    if not os.path.exists(cuda_lib):
        cuda_lib = os.path.join(os.path.dirname(inc), "lib")
    exe = tmp_path / "driver"
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.dirname(HDR), "-I", inc,
                        os.path.join(ROOT, "tests", "host_layer_driver.cpp"), "-o", str(exe),
                        "-L", lib_dir, "-lrigc", "-L", cuda_lib, "-lcudart",
                        f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{cuda_lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sc = S.scene_from_json(S.spec_cubes(0))
    x0 = contact_poses(sc)
    x1 = sc.predictor_poses(x0)
    dhat = 1e-3
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        for key, dt in (("rest_vertices", np.float64), ("edges", np.int32), ("faces", np.int32),
                        ("faces_to_edges", np.int32), ("body_vertex_start", np.int32),
                        ("body_edge_start", np.int32), ("body_face_start", np.int32),
                        ("group_ids", np.int32), ("body_type", np.int32),
                        ("r_max", np.float64)):
            _write_vec(f, getattr(sc, key), dt)
        _write_vec(f, [sc.average_edge_length], np.float64)
        _write_vec(f, x0, np.float64)
        _write_vec(f, x1, np.float64)
        _write_vec(f, [dhat], np.float64)
    r = subprocess.run([str(exe), str(inp), str(outp)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    with open(outp, "rb") as f:
        toi, e, md, isect, toi_pl, active = _read_vec(f, np.float64)
        g = _read_vec(f, np.float64)
        rp, col, val = _read_vec(f, np.int32), _read_vec(f, np.int32), _read_vec(f, np.float64)
        ee, fv = _read_vec(f, np.int32), _read_vec(f, np.int32)
    ctx = rigc.Context(sc)
    assert toi == ctx.compute_earliest_toi(x0, x1)
    assert toi_pl == ctx.compute_earliest_toi_piecewise_linear(x0, x1)
    assert active == (1.0 if np.isfinite(toi) else 0.0)
    ctx.construct_constraint_set(x0, dhat)
    e2, g2, (rp2, col2, val2) = ctx.compute_barrier_term(x0, dhat)
    assert e == e2 and np.array_equal(g, g2)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
    assert np.array_equal(val, np.asarray(val2).reshape(-1))
    ee2, fv2 = ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    assert np.array_equal(ee, ee2.reshape(-1)) and np.array_equal(fv, fv2.reshape(-1))
    assert md == ctx.compute_min_distance(x0, dhat) and md > 0
    assert isect == 0.0
