"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bars: candidate sets, constraint sets, world vertices and times of impact are
bit-exact (integer / decision work and the same round-to-nearest operation
order); barrier energy and gradient within 1e-10 relative, Hessians within
1e-9 relative (Frobenius, per local 12x12 or per assembled block row).
"""
import math

import numpy as np
import pytest

from test_oracle_pins import (EE_Y1, EE_Z, FV_Y, FV_Z1, PARALLEL_CASES, ee_case, fv_case,
                              parallel_edges)

pytestmark = pytest.mark.gpu

ENERGY_RTOL = 1e-10
GRAD_RTOL = 1e-10
HESS_RTOL = 1e-9


@pytest.fixture(scope="module")
def ctx_c1(cube_scene):
    import rigc

    return rigc.Context(cube_scene)


def _canon_constraints(types, verts, prims, bodies, weight, eps):
    """Order constraints by (type, prim0, prim1); VV by (min, max) vertex."""
    types = np.asarray(types)
    verts = np.array(verts)
    prims = np.array(prims)
    bodies = np.array(bodies)
    vv = types == 0
    swap = vv & (verts[:, 0] > verts[:, 1])
    verts[swap, 0], verts[swap, 1] = verts[swap, 1].copy(), verts[swap, 0].copy()
    bodies[swap, 0], bodies[swap, 1] = bodies[swap, 1].copy(), bodies[swap, 0].copy()
    prims[vv, 0], prims[vv, 1] = verts[vv, 0], verts[vv, 1]
    order = np.lexsort((prims[:, 1], prims[:, 0], types))
    return (types[order], verts[order], prims[order], bodies[order],
            np.asarray(weight)[order], np.asarray(eps)[order])


def test_world_vertices_bitexact(oracle, cube_scene, ctx_c1):
    rng = np.random.default_rng(1)
    o = oracle.OracleScene(cube_scene)
    for _ in range(3):
        x = cube_scene.poses() + rng.normal(0, 0.3, 6 * cube_scene.num_bodies)
        Vg = ctx_c1.world_vertices(x).cpu().numpy()
        Vo = o.world_vertices(x)
        assert np.array_equal(Vg, Vo)


@pytest.mark.parametrize("continuous", [False, True])
def test_candidates_bitexact(oracle, cube_scene, cube_contact, ctx_c1, continuous):
    o = oracle.OracleScene(cube_scene)
    x0 = cube_contact
    x1 = cube_scene.predictor_poses(x0) if continuous else x0
    infl = 0.0 if continuous else 5e-4
    ee_g, fv_g = ctx_c1.detect_collision_candidates_rigid(x0, x1, continuous, infl)
    ee_o, fv_o = o.detect_candidates(x0, x1, continuous, infl)
    ee_b, fv_b = o.detect_candidates(x0, x1, continuous, infl, brute=True)
    assert len(ee_o) > 0 and len(fv_o) > 0
    assert np.array_equal(ee_o, ee_b) and np.array_equal(fv_o, fv_b)
    assert np.array_equal(ee_g, ee_o)
    assert np.array_equal(fv_g, fv_o)


def test_constraint_set_bitexact(oracle, cube_scene, cube_contact, ctx_c1):
    dhat = 1e-3
    o = oracle.OracleScene(cube_scene)
    ee, fv = o.detect_candidates(cube_contact, continuous=False, inflation=dhat / 2)
    co = o.constraint_set(cube_contact, ee, fv, dhat)
    cg = ctx_c1.construct_constraint_set(cube_contact, dhat)
    assert len(co) > 0
    a = _canon_constraints(co.types, co.verts, co.prims, co.bodies, co.weight, co.eps)
    b = _canon_constraints(cg["type"], cg["verts"], cg["prims"], cg["bodies"], cg["weight"],
                           cg["eps"])
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def _rel_err(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


@pytest.mark.parametrize("project", [False, True])
def test_barrier_local_terms(oracle, cube_scene, cube_contact, ctx_c1, project):
    dhat = 1e-3
    o = oracle.OracleScene(cube_scene)
    ee, fv = o.detect_candidates(cube_contact, continuous=False, inflation=dhat / 2)
    cs = o.constraint_set(cube_contact, ee, fv, dhat)
    ctx_c1.set_constraints(cs.types, cs.verts, cs.prims, cs.bodies, cs.weight, cs.eps)
    e_o, g_o, H_o = o.local_terms(cube_contact, cs, dhat, project=project)
    e_g, g_g, H_g = ctx_c1.barrier_local_terms(cube_contact, len(cs), dhat, project=project)
    for i in range(len(cs)):
        assert abs(e_g[i] - e_o[i]) <= ENERGY_RTOL * abs(e_o[i])
        assert _rel_err(g_g[i], g_o[i]) <= GRAD_RTOL
        assert np.linalg.norm(H_g[i] - H_o[i]) <= HESS_RTOL * np.linalg.norm(H_o[i])


@pytest.mark.parametrize("project", [False, True])
@pytest.mark.parametrize("case", sorted(PARALLEL_CASES))
def test_barrier_mollified_ee_endpoint(oracle, case, project):
    """Near-parallel EE constraints whose closest features are endpoints
    (closest-feature distance with the mollifier) against the oracle."""
    import rigc

    sc = parallel_edges(PARALLEL_CASES[case])
    o = oracle.OracleScene(sc)
    x = np.zeros(12)
    x[9:12] = [1e-6, -2e-6, 1.5e-6]
    ee, fv = o.detect_candidates(x, continuous=False, inflation=5e-4)
    cs = o.constraint_set(x, ee, fv, 1e-3)
    assert list(cs.types) == [2]
    ctx = rigc.Context(sc)
    ctx.set_constraints(cs.types, cs.verts, cs.prims, cs.bodies, cs.weight, cs.eps)
    e_o, g_o, H_o = o.local_terms(x, cs, 1e-3, project=project)
    e_g, g_g, H_g = ctx.barrier_local_terms(x, len(cs), 1e-3, project=project)
    assert abs(e_g[0] - e_o[0]) <= ENERGY_RTOL * abs(e_o[0])
    assert _rel_err(g_g[0], g_o[0]) <= GRAD_RTOL
    assert np.linalg.norm(H_g[0] - H_o[0]) <= HESS_RTOL * np.linalg.norm(H_o[0])


def test_barrier_term_assembled(oracle, cube_scene, cube_contact, ctx_c1):
    dhat = 1e-3
    o = oracle.OracleScene(cube_scene)
    ee, fv = o.detect_candidates(cube_contact, continuous=False, inflation=dhat / 2)
    cs = o.constraint_set(cube_contact, ee, fv, dhat)
    e_o, g_o, (rp_o, col_o, val_o) = o.barrier_term(cube_contact, cs, dhat)
    # the GPU builds its own constraint set (bit-exact with the oracle's)
    ctx_c1.construct_constraint_set(cube_contact, dhat)
    e_g, g_g, (rp_g, col_g, val_g) = ctx_c1.compute_barrier_term(cube_contact, dhat)
    assert abs(e_g - e_o) <= ENERGY_RTOL * abs(e_o)
    assert _rel_err(g_g, g_o) <= GRAD_RTOL
    assert np.array_equal(rp_g, rp_o) and np.array_equal(col_g, col_o)
    for r in range(len(rp_o) - 1):
        blk_o = val_o[rp_o[r]:rp_o[r + 1]]
        blk_g = val_g[rp_o[r]:rp_o[r + 1]]
        if blk_o.size:
            assert np.linalg.norm(blk_g - blk_o) <= HESS_RTOL * max(np.linalg.norm(blk_o), 1e-300)


def _gpu_toi_case(sc, x0, x1, tol=1e-6):
    import rigc

    ctx = rigc.Context(sc)
    ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    toi, per, st = ctx.earliest_toi(x0, x1, toi_tol=tol, prune=False, per_candidate=True)
    return ctx, toi, per


@pytest.mark.parametrize("z", EE_Z)
@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("y_t1", [1.0, 0.1, 0.0, -1e-6, -2, -1000])
def test_gpu_edge_edge_toi_analytic(oracle, z, sign, y_t1):
    sc, x0, x1, expected, hit = ee_case(z, sign, y_t1)
    import rigc

    ctx = rigc.Context(sc)
    o = oracle.OracleScene(sc)
    ee_g, fv_g = ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    ee_o, fv_o = o.detect_candidates(x0, x1, True, 0.0)
    assert np.array_equal(ee_g, ee_o) and np.array_equal(fv_g, fv_o)
    toi_g = ctx.earliest_toi(x0, x1, toi_tol=1e-6, prune=False)
    if len(ee_g):
        is_hit_o, toi_o, _ = o.edge_edge_toi(x0, x1, 0, 1, bound=1.0, tol=1e-6)
        assert is_hit_o == hit
        assert math.isinf(toi_g) == (not is_hit_o)
        if is_hit_o:
            assert toi_g == toi_o
            assert toi_g <= expected
    else:
        assert not hit


@pytest.mark.parametrize("y", FV_Y)
@pytest.mark.parametrize("z_t1", FV_Z1)
def test_gpu_face_vertex_toi_analytic(oracle, y, z_t1):
    sc, x0, x1, expected, hit = fv_case(y, z_t1)
    import rigc

    ctx = rigc.Context(sc)
    o = oracle.OracleScene(sc)
    ee_g, fv_g = ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    toi_g, per, st = ctx.earliest_toi(x0, x1, toi_tol=1e-6, prune=False, per_candidate=True)
    toi_min, per_o, _ = o.earliest_toi(x0, x1, ee_g, fv_g, tol=1e-6, per_candidate=True)
    assert toi_g == toi_min
    assert np.array_equal(per, per_o)
    if hit:
        assert toi_g <= expected
        assert toi_g == pytest.approx(expected, abs=1e-4)


def test_ccd_per_candidate_bitexact(oracle, cube_scene, cube_contact, ctx_c1):
    x0 = cube_contact
    x1 = cube_scene.predictor_poses(x0)
    o = oracle.OracleScene(cube_scene)
    ee, fv = ctx_c1.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    toi_o, per_o, _ = o.earliest_toi(x0, x1, ee, fv, per_candidate=True, nthreads=8)
    toi_g, per_g, st = ctx_c1.earliest_toi(x0, x1, prune=False, per_candidate=True)
    assert st == 0
    assert np.array_equal(per_g, per_o)
    assert toi_g == toi_o
    # pruned search: same earliest time of impact
    toi_p = ctx_c1.earliest_toi(x0, x1, prune=True)
    assert toi_p == toi_o
    assert ctx_c1.compute_earliest_toi(x0, x1) == toi_o


def test_narrow_phase_host_matches_device(cube_scene, cube_contact, ctx_c1):
    x0 = cube_contact
    x1 = cube_scene.predictor_poses(x0)
    dhat = 1e-3
    toi, energy, grad, (rp, col, val), nnzb = ctx_c1.narrow_phase_host(x0, x1, dhat)
    assert toi == ctx_c1.compute_earliest_toi(x0, x1)
    ctx_c1.construct_constraint_set(x0, dhat)
    e2, g2, (rp2, col2, val2) = ctx_c1.compute_barrier_term(x0, dhat)
    assert energy == e2 and np.array_equal(grad, g2)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2) and np.array_equal(val, val2)


def test_body_energy(oracle, cube_scene, cube_contact, ctx_c1):
    """compute_energy_term per body vs the oracle's autodiff restatement."""
    sc = cube_scene
    rng = np.random.default_rng(3)
    x = cube_contact + rng.normal(0, 0.05, 6 * sc.num_bodies)
    e_g, g_g, H_g = ctx_c1.body_energy(x)
    e_sum = 0.0
    for b, body in enumerate(sc.bodies):
        e_o, g_o, H_o = oracle.body_energy(body, x[6 * b:6 * b + 6], sc.gravity, sc.timestep)
        e_sum += e_o
        assert np.abs(g_g[6 * b:6 * b + 6] - g_o).max() <= GRAD_RTOL * max(np.abs(g_o).max(), 1.0)
        assert np.linalg.norm(H_g[b] - H_o) <= HESS_RTOL * max(np.linalg.norm(H_o), 1.0)
    assert abs(e_g - e_sum) <= ENERGY_RTOL * max(abs(e_sum), 1.0)


def test_error_statuses(cube_scene, ctx_c1):
    import ctypes as C

    import rigc
    from rigc import _lib as L

    lib = L.load()
    assert lib.rigc_ctx_create(None, None) == L.RIGC_ERR_ARG
    assert lib.rigc_barrier_term(ctx_c1.h, None, 1e-3, 0.0, 3, None) == L.RIGC_ERR_ARG
    x = cube_scene.poses()
    x[3] = np.nan
    with pytest.raises(L.RigcError) as e:
        ctx_c1.narrow_phase_host(x, x, 1e-3)
    assert e.value.status == L.RIGC_ERR_NAN


def test_chain_links_parity(oracle):
    """Three links of the hanging chain (interlocked 48 x 24 tori with a 1 mm
    gap, the edge-edge-dominated configuration; dhat 2e-3 so that the links
    are in the constraint set): candidate sets, per-candidate times of impact
    (a box budget of 2^14, the same on both sides), the constraint set and
    the barrier term against the oracle."""
    import rigc
    from rigc import scene as S

    sc = S.scene_from_json(S.spec_chain(3, spacing=1.499))
    o = oracle.OracleScene(sc)
    x0 = sc.poses()
    x1 = x0.reshape(-1, 6).copy()
    x1[1:, 1] -= 9.81 * 0.005 ** 2
    x1[2, 4] += 1e-3  # and a small turn of the last link
    x1 = x1.reshape(-1)
    ctx = rigc.Context(sc)
    ee_g, fv_g = ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    ee_o, fv_o = o.detect_candidates(x0, x1, True, 0.0)
    assert len(ee_o) > 100 and np.array_equal(ee_g, ee_o) and np.array_equal(fv_g, fv_o)
    budget = 1 << 14
    ctx.set_ccd_budget(budget)
    toi_o, per_o, _, st_o = o.earliest_toi(x0, x1, ee_o, fv_o, per_candidate=True, nthreads=8,
                                           max_boxes=budget, with_status=True)
    toi_g, per_g, st_g = ctx.earliest_toi(x0, x1, prune=False, per_candidate=True)
    assert np.array_equal(per_g, per_o) and toi_g == toi_o and st_g == st_o
    dhat = 2e-3
    cs = ctx.construct_constraint_set(x0, dhat)
    ee, fv = o.detect_candidates(x0, continuous=False, inflation=dhat / 2)
    cs_o = o.constraint_set(x0, ee, fv, dhat)
    assert len(cs_o) > 0
    a = _canon_constraints(cs_o.types, cs_o.verts, cs_o.prims, cs_o.bodies, cs_o.weight, cs_o.eps)
    b = _canon_constraints(cs["type"], cs["verts"], cs["prims"], cs["bodies"], cs["weight"],
                           cs["eps"])
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    e_g, g_g, _ = ctx.compute_barrier_term(x0, dhat)
    e_o, g_o, _ = o.barrier_term(x0, cs_o, dhat)
    assert abs(e_g - e_o) <= ENERGY_RTOL * abs(e_o)
    assert _rel_err(g_g, g_o) <= GRAD_RTOL


def test_min_distance(oracle, cube_scene, cube_contact, ctx_c1):
    """compute_min_distance at the stacked contact (constraints present) and
    at the lattice poses (no constraint: -1) against the oracle; the minimum
    is bit-exact (the same round-to-nearest distances, a min)."""
    dhat = 1e-3
    o = oracle.OracleScene(cube_scene)
    d_o = o.min_distance(cube_contact, dhat)
    d_g = ctx_c1.compute_min_distance(cube_contact, dhat)
    assert 0 < d_o < dhat
    assert d_g == d_o
    x = cube_scene.poses()
    assert o.min_distance(x, dhat) == -1
    assert ctx_c1.compute_min_distance(x, dhat) == -1
    # with dmin the set grows (inflation (dhat + dmin) / 2) and the same
    # distances enter it
    assert ctx_c1.compute_min_distance(cube_contact, dhat, 2e-4) == o.min_distance(
        cube_contact, dhat, 2e-4)
