"""Batched contexts (rigc_ctx_create_batched): independent scenes in one
context give exactly the per-scene results of one context per scene --
candidate sets (with index offsets), per-scene earliest times of impact,
constraint sets, per-scene barrier energies (1e-12: summed in another order)
and the gradient (bit for bit)."""
import os

import numpy as np
import pytest

from conftest import contact_poses

pytestmark = pytest.mark.gpu

DHAT = 1e-3
ENERGY_RTOL = 1e-10


def _scenes():
    from rigc import scene as S

    out = []
    for seed in (0, 1, 2):
        sc = S.scene_from_json(S.spec_cubes(seed))
        out.append((sc, contact_poses(sc, seed=seed)))
    return out


def test_batched_matches_plain():
    import rigc
    from rigc import scene as S

    items = _scenes()
    big, sob = S.concat_scenes([sc for sc, _ in items])
    x0 = np.concatenate([x for _, x in items])
    x1 = np.concatenate([sc.predictor_poses(x) for sc, x in items])
    cb = rigc.Context(big, scene_of_body=sob)
    ee_b, fv_b = cb.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    toi_b = cb.compute_earliest_toi(x0, x1)
    scene_toi = cb.scene_tois()
    cs_b = cb.construct_constraint_set(x0, DHAT)
    e_b, g_b, _ = cb.compute_barrier_term(x0, DHAT)
    se_b = cb.scene_barrier_energies()

    ee_p, fv_p, tois, grads, energies, ncons = [], [], [], [], [], 0
    vo = eo = fo = 0
    for sc, x in items:
        cp = rigc.Context(sc)
        x1s = sc.predictor_poses(x)
        ee, fv = cp.detect_collision_candidates_rigid(x, x1s, True, 0.0)
        ee_p.append(ee + eo)
        fv_p.append(fv + np.array([fo, vo]))
        tois.append(cp.compute_earliest_toi(x, x1s))
        cs = cp.construct_constraint_set(x, DHAT)
        ncons += len(cs["type"])
        e, g, _ = cp.compute_barrier_term(x, DHAT)
        energies.append(e)
        grads.append(g)
        vo += sc.num_vertices
        eo += len(sc.edges)
        fo += len(sc.faces)
    assert len(ee_b) > 0 and len(fv_b) > 0
    assert np.array_equal(ee_b, np.concatenate(ee_p))
    assert np.array_equal(fv_b, np.concatenate(fv_p))
    assert np.array_equal(scene_toi, np.array(tois))
    assert toi_b == min(tois)
    assert len(cs_b["type"]) == ncons
    assert np.array_equal(g_b, np.concatenate(grads))
    assert np.allclose(se_b, energies, rtol=1e-12, atol=0)
    assert e_b == pytest.approx(sum(energies), rel=1e-12)


def _contact_pairs():
    """Small contact scenes (two cubes landing on a plane, the second sliding
    into the first) with different seeded rotations and spins."""
    from rigc import scene as S

    from test_adjoint_oracle import contact_pair_spec

    return [S.scene_from_json(contact_pair_spec(seed)) for seed in (3, 4, 5, 6)]


def test_batched_sim_matches_plain():
    """rigc_sim_step on a batched context steps every scene as its own
    problem: the poses and velocities after 6 contact steps equal those of
    one context per scene up to the linear-solve accuracy (the batched path
    solves each scene's Newton system by PCG, the plain one factorises it)."""
    import rigc
    from rigc import scene as S

    scenes = _contact_pairs()
    steps = 6
    plain = []
    for sc in scenes:
        ctx = rigc.Context(sc)
        ctx.sim_init(0.01, (0.0, -9.81, 0.0), DHAT)
        st = ctx.sim_step(steps)
        P, V, Q, k = ctx.sim_state()
        plain.append((P, V, st["newton_iterations"]))
    big, sob = S.concat_scenes(scenes)
    cb = rigc.Context(big, scene_of_body=sob)
    cb.sim_init(0.01, (0.0, -9.81, 0.0), DHAT)
    st_b = cb.sim_step(steps)
    P, V, Q, k = cb.sim_state()
    vs = np.r_[0, np.cumsum([sc.num_bodies for sc in scenes])]
    for i, (Pp, Vp, it) in enumerate(plain):
        assert np.abs(P[vs[i]:vs[i + 1]] - Pp).max() <= 1e-8
        assert np.abs(V[vs[i]:vs[i + 1]] - Vp).max() <= 1e-6
    # the batched count is per scene: the sum of the plain ones
    assert st_b["newton_iterations"] == sum(it for _, _, it in plain)


def test_batched_sim_rejects_friction():
    import rigc
    from rigc import scene as S

    big, sob = S.concat_scenes(_contact_pairs()[:2])
    cb = rigc.Context(big, scene_of_body=sob)
    cb.sim_init(0.01, (0.0, -9.81, 0.0), DHAT, coefficient_friction=0.5)
    with pytest.raises(RuntimeError):
        cb.sim_step(1)


def test_autotune_keeps_results():
    """rigc_autotune only changes launch shapes: the earliest times of impact
    (per scene), the constraint set and the barrier term are the same after
    it, bit for bit."""
    import rigc
    from rigc import scene as S

    items = _scenes()
    big, sob = S.concat_scenes([sc for sc, _ in items])
    x0 = np.concatenate([x for _, x in items])
    x1 = np.concatenate([sc.predictor_poses(x) for sc, x in items])
    cb = rigc.Context(big, scene_of_body=sob)

    def run():
        toi = cb.compute_earliest_toi(x0, x1)
        st = cb.scene_tois()
        cs = cb.construct_constraint_set(x0, DHAT)
        e, g, _ = cb.compute_barrier_term(x0, DHAT)
        return toi, st, cs, e, g

    a = run()
    rep = cb.autotune(x0, x1, DHAT)
    assert rep["ccd_ms"] <= rep["ccd_ms_default"] and rep["barrier_ms"] <= rep["barrier_ms_default"]
    b = run()
    assert a[0] == b[0] and np.array_equal(a[1], b[1])
    for k in a[2]:
        assert np.array_equal(np.asarray(a[2][k]), np.asarray(b[2][k])), k
    assert a[3] == b[3] and np.array_equal(a[4], b[4])
    cb.set_tune(1, 256, 4, 3)
    c = run()
    assert a[0] == c[0] and a[3] == c[3] and np.array_equal(a[4], c[4])


def test_batched_hull_scenes_match_oracle(oracle):
    """Eight scenes of the batched benchmark (convex hulls of 32 random
    unit-sphere points in seeded piles on their own planes, bench._hull_scene)
    in one batched context, each scene against the oracle run on that scene
    alone: continuous and discrete candidate sets and per-scene earliest
    times of impact bit for bit, constraint sets bit for bit, per-scene
    barrier energies and the gradient to 1e-10."""
    import bench
    import rigc
    from rigc import scene as S

    from test_gpu_parity import _canon_constraints

    items = [bench._hull_scene(10_000 + k) for k in range(8)]
    scenes = [sc for sc, _, _ in items]
    big, sob = S.concat_scenes(scenes)
    X0 = np.concatenate([x for _, x, _ in items])
    X1 = np.concatenate([x for _, _, x in items])
    cb = rigc.Context(big, scene_of_body=sob)
    ee_b, fv_b = cb.detect_collision_candidates_rigid(X0, X1, True, 0.0)
    cb.compute_earliest_toi(X0, X1)
    tois_b = cb.scene_tois()
    # the CCD's time windows (per-scene running minima) change no bit
    for k in (0, 3, 12):
        cb.set_ccd_window(k)
        cb.compute_earliest_toi(X0, X1)
        assert np.array_equal(cb.scene_tois(), tois_b), k
    cb.set_ccd_window(-1)
    eed_b, fvd_b = cb.detect_collision_candidates_rigid(X0, X0, False, DHAT / 2)
    cs_b = cb.construct_constraint_set(X0, DHAT)
    e_b, g_b, _ = cb.compute_barrier_term(X0, DHAT)
    se_b = cb.scene_barrier_energies()

    ee_o, fv_o, eed_o, fvd_o, tois_o, grads_o, cons_o = [], [], [], [], [], [], []
    vo = eo = fo = bo = 0
    for sc, x0, x1 in items:
        o = oracle.OracleScene(sc)
        ee, fv = o.detect_candidates(x0, x1, True, 0.0)
        tois_o.append(o.earliest_toi(x0, x1, ee, fv, nthreads=os.cpu_count() or 1,
                                     max_boxes=1 << 22))
        ee_o.append(ee + eo)
        fv_o.append(fv + np.array([fo, vo]))
        eed, fvd = o.detect_candidates(x0, continuous=False, inflation=DHAT / 2)
        eed_o.append(eed + eo)
        fvd_o.append(fvd + np.array([fo, vo]))
        cs = o.constraint_set(x0, eed, fvd, DHAT)
        e, g, _ = o.barrier_term(x0, cs, DHAT)
        grads_o.append((e, g))
        # global indices: vertices, edges, faces and bodies after the
        # earlier scenes' (prims: VV (v, v), EV (e, v), EE (e, e), FV (f, v))
        prim_off = np.array([[vo, vo], [eo, vo], [eo, eo], [fo, vo]])[cs.types]
        cons_o.append((cs.types, np.where(cs.verts >= 0, cs.verts + vo, cs.verts),
                       cs.prims + prim_off, cs.bodies + bo, cs.weight, cs.eps))
        vo += sc.num_vertices
        eo += len(sc.edges)
        fo += len(sc.faces)
        bo += sc.num_bodies
    assert sum(len(e) for e in ee_o) > 0 and sum(len(f) for f in fv_o) > 0
    assert np.array_equal(ee_b, np.concatenate(ee_o))
    assert np.array_equal(fv_b, np.concatenate(fv_o))
    assert np.array_equal(eed_b, np.concatenate(eed_o))
    assert np.array_equal(fvd_b, np.concatenate(fvd_o))
    assert np.array_equal(tois_b, np.array(tois_o))
    a = _canon_constraints(*[np.concatenate([c[k] for c in cons_o]) for k in range(6)])
    b = _canon_constraints(cs_b["type"], cs_b["verts"], cs_b["prims"], cs_b["bodies"],
                           cs_b["weight"], cs_b["eps"])
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    for k, (e, g) in enumerate(grads_o):
        assert abs(se_b[k] - e) <= ENERGY_RTOL * max(abs(e), 1e-300)
    g_o = np.concatenate([g for _, g in grads_o])
    assert np.abs(g_b - g_o).max() <= ENERGY_RTOL * max(np.abs(g_o).max(), 1e-300)
