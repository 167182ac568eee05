"""The device piecewise-linear CCD (rigc_earliest_toi_piecewise_linear /
rigc_compute_earliest_toi_piecewise_linear through the C ABI) against the
oracle's restatement: per-candidate times of impact bit for bit on the
reference's 403 CCD queries, on the continuous candidates of the 575-body
wrecking-ball scene and of the 27-cube lattice's first step, and the
earliest time of impact of the whole broad + narrow phase."""
import numpy as np
import pytest

from test_reference_fixtures import queries, scene_fixture

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("per_lane", [0, 1])
def test_pl_reference_queries_gpu(per_lane):
    """All 403 queries in one context, candidates given explicitly, one
    candidate per warp and per lane."""
    import make_reference_fixtures as M
    import oracle as O
    import rigc
    from rigc import scene as S

    q = queries()
    bodies, ee, fv, expect = [], [], [], []
    nv = ne = nf = 0
    x0, x1 = [], []
    for k, V, P in zip(q["kind"], q["vertices"], q["poses"]):
        sc = M.query_scene(int(k), V)
        o = O.OracleScene(sc)
        p0 = np.concatenate([P[0, 0], P[1, 0]])
        p1 = np.concatenate([P[0, 1], P[1, 1]])
        hit, toi, _ = o.pl_toi(p0, p1, int(k), 0, 1 if k == 0 else 3)
        expect.append((int(k), toi))
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
    ctx = rigc.Context(S.Scene(bodies=bodies))
    ctx.set_pl_search(per_lane)
    ctx.set_candidates(ee, fv)
    toi, per, st = ctx.earliest_toi_piecewise_linear(np.concatenate(x0), np.concatenate(x1),
                                                     per_candidate=True)
    want = np.array([t for k, t in expect if k == 0] + [t for k, t in expect if k == 1])
    assert np.array_equal(per, want)
    assert toi == want.min() and st == 0
    assert np.isfinite(want).sum() > 100


@pytest.mark.parametrize("per_lane", [0, 1])
def test_pl_wrecking_ball_scene_gpu(oracle, per_lane):
    """The 66,536 continuous candidates of the 575-body wrecking-ball scene,
    one candidate per warp and per lane."""
    import make_reference_fixtures as M
    import rigc

    d = scene_fixture()
    sc = M.scene_from_fixture(d)
    x0 = d["pose_t0"].reshape(-1)
    x1 = d["pose_t1"].reshape(-1)
    ctx = rigc.Context(sc)
    ctx.set_pl_search(per_lane)
    ee, fv = ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    toi, per, st = ctx.earliest_toi_piecewise_linear(x0, x1, per_candidate=True)
    o = oracle.OracleScene(sc)
    t_o, per_o, st_o = o.pl_earliest_toi(x0, x1, ee, fv, nthreads=16)
    assert np.array_equal(per, per_o)
    assert toi == t_o and st == st_o["status"]


@pytest.mark.parametrize("dmin", [0.0, 1e-4])
def test_pl_cube_lattice_gpu(oracle, cube_scene, dmin):
    """The 27-cube lattice in contact (0.5 mm gaps) between its poses and the
    explicit step of its velocities: broad phase (inflation dmin / 2) and
    piecewise-linear narrow phase, per candidate and the earliest time."""
    import rigc
    from conftest import contact_poses

    x0 = contact_poses(cube_scene)
    x1 = cube_scene.predictor_poses(x0)
    ctx = rigc.Context(cube_scene)
    t_all = ctx.compute_earliest_toi_piecewise_linear(x0, x1, dmin)
    ee, fv = ctx.detect_collision_candidates_rigid(x0, x1, True, dmin / 2)
    toi, per, st = ctx.earliest_toi_piecewise_linear(x0, x1, dmin, per_candidate=True)
    o = oracle.OracleScene(cube_scene)
    t_o, per_o, _ = o.pl_earliest_toi(x0, x1, ee, fv, dmin=dmin, nthreads=16)
    assert np.array_equal(per, per_o)
    assert toi == t_o and t_all == t_o
