"""The CUDA path on the reference's own CCD test data (fixtures packed by
tests/golden/make_reference_fixtures.py, oracle results stored with them):
per-query and per-candidate times of impact bit-exact, the wrecking-ball
scene's candidate set identical, with one search per lane (k_ccd), one
per warp (k_ccd_group<32>, as compiled and fitted to 4 or 5 blocks per SM)
and one per half-warp (k_ccd_group<16>, as compiled and fitted to 4 blocks
per SM) alike."""
import os

import numpy as np
import pytest

from test_reference_fixtures import queries, scene_fixture

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("warp", [0, 1, 2, 3, 4, 5])
def test_reference_queries_gpu(warp):
    """All 403 queries in one context, candidates given explicitly."""
    import make_reference_fixtures as M
    import rigc
    from rigc import scene as S

    q = queries()
    bodies, ee, fv = [], [], []
    nv = ne = nf = 0
    x0, x1 = [], []
    for k, V, P in zip(q["kind"], q["vertices"], q["poses"]):
        sc = M.query_scene(int(k), V)
        for b in sc.bodies:
            b.group_id = len(bodies)
            bodies.append(b)
        a, b = sc.bodies
        if k == 0:
            ee.append((ne, ne + 1))
        else:
            fv.append((nf, nv + 3))
        for body in (a, b):
            nv += len(body.vertices)
            ne += len(body.edges)
            nf += len(body.faces)
        x0 += [P[0, 0], P[1, 0]]
        x1 += [P[0, 1], P[1, 1]]
    scene = S.Scene(bodies=bodies)
    ctx = rigc.Context(scene)
    ctx.set_tune(ccd_warp=warp)
    ctx.set_ccd_budget(int(q["budget"]))
    ctx.set_candidates(ee, fv)
    x0 = np.concatenate(x0)
    x1 = np.concatenate(x1)
    toi, per, st = ctx.earliest_toi(x0, x1, toi_tol=1e-4, prune=False, per_candidate=True)
    kinds = q["kind"]
    expect = np.concatenate([q["toi_oracle"][kinds == 0], q["toi_oracle"][kinds == 1]])
    assert np.array_equal(per, expect)
    assert st == 5  # the queries at t = 0 end at the budget
    assert toi == expect.min()


@pytest.mark.parametrize("warp", [0, 1, 2, 3, 4, 5])
def test_wrecking_ball_scene_gpu(warp):
    import make_reference_fixtures as M
    import rigc

    d = scene_fixture()
    sc = M.scene_from_fixture(d)
    ctx = rigc.Context(sc)
    ctx.set_tune(ccd_warp=warp)
    x0 = d["pose_t0"].reshape(-1)
    x1 = d["pose_t1"].reshape(-1)
    ee, fv = ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    assert len(ee) == int(d["num_ee"]) and len(fv) == int(d["num_fv"])
    assert M.candidates_digest(ee, fv) == str(d["candidates_sha256"])
    ctx.set_ccd_budget(int(d["budget"]))
    toi, per, st = ctx.earliest_toi(x0, x1, toi_tol=1e-4, prune=False, per_candidate=True)
    assert st == int(d["status_oracle"])
    idx = np.flatnonzero(np.isfinite(per))
    assert np.array_equal(idx, d["toi_idx"])
    assert np.array_equal(per[idx], d["toi_val"])
    assert toi == float(d["toi_min"])
    # With cross-candidate pruning the lanes of a warp share the last
    # searches; a search stopped by the box budget (here: bodies resting in
    # contact at t = 0) then reports a conservative bound that need not equal
    # the single-search one.  It stays at or below every time of impact the
    # oracle resolved exactly (the t.lo > 0 roots).
    toi_p = ctx.earliest_toi(x0, x1, toi_tol=1e-4, prune=True)
    exact = d["toi_val"][d["toi_val"] > 0]
    assert 0.0 <= toi_p <= exact.min()
