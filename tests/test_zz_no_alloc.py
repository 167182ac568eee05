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


def _stacked_case(oracle, S, rigc, n):
    """The n x n x n cube lattice with every column stacked on the floor
    (cubes within the barrier distance of the one below), its constraint set
    and two pose sets."""
    sc = S.scene_from_json(S.spec_cubes(0, n=n))
    ctx = rigc.Context(sc)
    o = oracle.OracleScene(sc)
    x_a = contact_poses(sc, seed=0)
    x_b = contact_poses(sc, seed=1)
    dhat = 1e-3
    ee, fv = o.detect_candidates(x_a, continuous=False, inflation=dhat / 2)
    cs = o.constraint_set(x_a, ee, fv, dhat)
    assert len(cs) > 0
    return sc, ctx, cs, (x_a, x_b), dhat


@pytest.fixture(scope="module")
def setup():
    import torch

    import oracle
    import rigc
    from rigc import scene as S

    oracle.build()
    sc, ctx, cs, poses, dhat = _stacked_case(oracle, S, rigc, 3)
    return torch, rigc, sc, ctx, cs, poses, dhat


@pytest.fixture(scope="module")
def large():
    """512 stacked cubes and the floor: 513 bodies, hundreds of constraints."""
    import oracle
    import rigc
    from rigc import scene as S

    oracle.build()
    return _stacked_case(oracle, S, rigc, 8)


def _noalloc(torch, rigc, sc, cs, x, dhat, flags, types=None, verts=None, bodies=None):
    lib = rigc.L.load()
    dev = dict(device="cuda")
    rest = torch.as_tensor(np.ascontiguousarray(sc.rest_vertices), dtype=torch.float64, **dev)
    xd = torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, **dev)
    t = torch.as_tensor(cs.types if types is None else types, dtype=torch.int32, **dev)
    v = torch.as_tensor(cs.verts if verts is None else verts, dtype=torch.int32, **dev)
    b = torch.as_tensor(cs.bodies if bodies is None else bodies, dtype=torch.int32, **dev)
    w = torch.as_tensor(cs.weight, dtype=torch.float64, **dev)
    e_x = torch.as_tensor(cs.eps, dtype=torch.float64, **dev)
    n = len(cs)
    energy = torch.full((n,), np.nan, dtype=torch.float64, **dev)
    grad = torch.full((n, 12), np.nan, dtype=torch.float64, **dev)
    hess = torch.full((n, 12, 12), np.nan, dtype=torch.float64, **dev)
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.rigc_barrier_local_terms_noalloc(
        rest.data_ptr(), len(sc.rest_vertices), sc.num_bodies, xd.data_ptr(), n, t.data_ptr(), v.data_ptr(),
        b.data_ptr(), w.data_ptr(), e_x.data_ptr(), dhat, 0.0, flags, energy.data_ptr(),
        grad.data_ptr(), hess.data_ptr(), C.c_void_p(stream))
    assert st == 0, lib.rigc_status_string(st)
    torch.cuda.synchronize()
    return energy.cpu().numpy(), grad.cpu().numpy(), hess.cpu().numpy()


def _check_against_regular(torch, rigc, sc, ctx, cs, x, dhat, project):
    flags = rigc.L.RIGC_GRAD | rigc.L.RIGC_HESS | (rigc.L.RIGC_PROJECT_PSD if project else 0)
    ctx.set_constraints(cs.types, cs.verts, cs.prims, cs.bodies, cs.weight, cs.eps)
    e_r, g_r, H_r = ctx.barrier_local_terms(x, len(cs), dhat, project=project)
    e_n, g_n, H_n = _noalloc(torch, rigc, sc, cs, x, dhat, flags)
    assert np.all(np.isfinite(e_n))
    assert np.all(np.abs(e_n - e_r) <= ENERGY_RTOL * np.abs(e_r))
    gs = np.maximum(np.abs(g_r).max(axis=1), 1e-300)
    assert np.all(np.abs(g_n - g_r).max(axis=1) <= GRAD_RTOL * gs)
    hs = np.maximum(np.linalg.norm(H_r, axis=(1, 2)), 1e-300)
    assert np.all(np.linalg.norm(H_n - H_r, axis=(1, 2)) <= HESS_RTOL * hs)


@pytest.mark.parametrize("project", [False, True])
def test_noalloc_matches_regular_entry_point(setup, project):
    torch, rigc, sc, ctx, cs, poses, dhat = setup
    # two calls in a row on different poses: the shared working array must
    # not carry the first call's frames into the second
    for x in poses:
        _check_against_regular(torch, rigc, sc, ctx, cs, x, dhat, project)


def test_noalloc_large_then_small(setup, large):
    """A call on 513 bodies, then one on 28: the second must not read the
    frames the first left in the shared array past its own bodies."""
    torch, rigc, sc, ctx, cs, poses, dhat = setup
    sc_l, ctx_l, cs_l, poses_l, _ = large
    assert sc_l.num_bodies > 500 and len(cs_l) > 300
    _check_against_regular(torch, rigc, sc_l, ctx_l, cs_l, poses_l[0], dhat, True)
    _check_against_regular(torch, rigc, sc, ctx, cs, poses[1], dhat, True)
    _check_against_regular(torch, rigc, sc_l, ctx_l, cs_l, poses_l[1], dhat, False)


def test_noalloc_out_of_range_indices_give_nan(setup):
    """Constraints whose body or vertex index is out of range (or whose type
    is unknown) read nothing and get NaN outputs; the others are unchanged."""
    torch, rigc, sc, ctx, cs, poses, dhat = setup
    flags = rigc.L.RIGC_GRAD | rigc.L.RIGC_HESS
    types = np.array(cs.types, dtype=np.int32)
    verts = np.array(cs.verts, dtype=np.int32).reshape(len(cs), 4)
    bodies = np.array(cs.bodies, dtype=np.int32).reshape(len(cs), 2)
    bad = [0, 1, 2, 3] if len(cs) > 4 else [0]
    bodies[bad[0], 1] = sc.num_bodies
    if len(bad) > 1:
        verts[bad[1], 0] = len(sc.rest_vertices)
        bodies[bad[2], 0] = -1
        types[bad[3]] = 7
    e_n, g_n, H_n = _noalloc(torch, rigc, sc, cs, poses[0], dhat, flags, types=types,
                             verts=verts.reshape(-1), bodies=bodies.reshape(-1))
    ctx.set_constraints(cs.types, cs.verts, cs.prims, cs.bodies, cs.weight, cs.eps)
    e_r, g_r, H_r = ctx.barrier_local_terms(poses[0], len(cs), dhat, project=False)
    for i in range(len(cs)):
        if i in bad:
            assert np.isnan(e_n[i]) and np.all(np.isnan(g_n[i])) and np.all(np.isnan(H_n[i]))
        else:
            assert abs(e_n[i] - e_r[i]) <= ENERGY_RTOL * abs(e_r[i])


def test_noalloc_rejects_too_many_bodies(setup):
    torch, rigc, sc, ctx, cs, poses, dhat = setup
    lib = rigc.L.load()
    st = lib.rigc_barrier_local_terms_noalloc(
        None, 0, rigc.L.RIGC_NOALLOC_MAX_BODIES + 1, None, 0, None, None, None, None, None,
        dhat, 0.0, rigc.L.RIGC_GRAD, None, None, None, None)
    assert st == rigc.L.RIGC_ERR_TOO_LARGE
    assert b"capacity" in lib.rigc_status_string(st)
