"""The entry point that allocates nothing, checked against the regular one.

rigc_barrier_local_terms_noalloc serves callers that cannot allocate device
memory at call time (a plugin inside a host application that owns the GPU's
memory, or a latency-critical loop where cudaMalloc would synchronise the
device): they pass every input and output as device memory they own, and the
library's only working memory is a fixed device array of
RIGC_NOALLOC_MAX_BODIES body frames.  This file is collected last so that a
run stopping at the first failure has already run every other test; it
creates all its state itself, so it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import contact_poses

pytestmark = pytest.mark.gpu

ENERGY_RTOL = 1e-10
GRAD_RTOL = 1e-10
HESS_RTOL = 1e-9


@pytest.fixture(scope="module")
def setup():
    import torch

    import oracle
    import rigc
    from rigc import scene as S

    oracle.build()
    sc = S.scene_from_json(S.spec_cubes(0))
    ctx = rigc.Context(sc)
    o = oracle.OracleScene(sc)
    x_a = contact_poses(sc, seed=0)
    x_b = contact_poses(sc, seed=1)
    dhat = 1e-3
    ee, fv = o.detect_candidates(x_a, continuous=False, inflation=dhat / 2)
    cs = o.constraint_set(x_a, ee, fv, dhat)
    assert len(cs) > 0
    return torch, rigc, sc, ctx, cs, (x_a, x_b), dhat


def _noalloc(torch, rigc, sc, cs, x, dhat, flags):
    lib = rigc.L.load()
    dev = dict(device="cuda")
    rest = torch.as_tensor(np.ascontiguousarray(sc.rest_vertices), dtype=torch.float64, **dev)
    xd = torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, **dev)
    t = torch.as_tensor(cs.types, dtype=torch.int32, **dev)
    v = torch.as_tensor(cs.verts, dtype=torch.int32, **dev)
    b = torch.as_tensor(cs.bodies, dtype=torch.int32, **dev)
    w = torch.as_tensor(cs.weight, dtype=torch.float64, **dev)
    e_x = torch.as_tensor(cs.eps, dtype=torch.float64, **dev)
    n = len(cs)
    energy = torch.full((n,), np.nan, dtype=torch.float64, **dev)
    grad = torch.full((n, 12), np.nan, dtype=torch.float64, **dev)
    hess = torch.full((n, 12, 12), np.nan, dtype=torch.float64, **dev)
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.rigc_barrier_local_terms_noalloc(
        rest.data_ptr(), sc.num_bodies, xd.data_ptr(), n, t.data_ptr(), v.data_ptr(),
        b.data_ptr(), w.data_ptr(), e_x.data_ptr(), dhat, 0.0, flags, energy.data_ptr(),
        grad.data_ptr(), hess.data_ptr(), C.c_void_p(stream))
    assert st == 0, lib.rigc_status_string(st)
    torch.cuda.synchronize()
    return energy.cpu().numpy(), grad.cpu().numpy(), hess.cpu().numpy()


@pytest.mark.parametrize("project", [False, True])
def test_noalloc_matches_regular_entry_point(setup, project):
    torch, rigc, sc, ctx, cs, poses, dhat = setup
    flags = rigc.L.RIGC_GRAD | rigc.L.RIGC_HESS | (rigc.L.RIGC_PROJECT_PSD if project else 0)
    ctx.set_constraints(cs.types, cs.verts, cs.prims, cs.bodies, cs.weight, cs.eps)
    # two calls in a row on different poses: the shared working array must
    # not carry the first call's frames into the second
    for x in poses:
        e_r, g_r, H_r = ctx.barrier_local_terms(x, len(cs), dhat, project=project)
        e_n, g_n, H_n = _noalloc(torch, rigc, sc, cs, x, dhat, flags)
        assert np.all(np.isfinite(e_n))
        for i in range(len(cs)):
            assert abs(e_n[i] - e_r[i]) <= ENERGY_RTOL * abs(e_r[i])
            scale = max(np.abs(g_r[i]).max(), 1e-300)
            assert np.abs(g_n[i] - g_r[i]).max() <= GRAD_RTOL * scale
            assert np.linalg.norm(H_n[i] - H_r[i]) <= HESS_RTOL * max(np.linalg.norm(H_r[i]), 1e-300)


def test_noalloc_rejects_too_many_bodies(setup):
    torch, rigc, sc, ctx, cs, poses, dhat = setup
    lib = rigc.L.load()
    st = lib.rigc_barrier_local_terms_noalloc(
        None, rigc.L.RIGC_NOALLOC_MAX_BODIES + 1, None, 0, None, None, None, None, None,
        dhat, 0.0, rigc.L.RIGC_GRAD, None, None, None, None)
    assert st == rigc.L.RIGC_ERR_TOO_LARGE
    assert b"capacity" in lib.rigc_status_string(st)
