"""Pins of the CPU oracle against the reference's own tests.

Each case restates a test of the rigid-ipc suite with its inputs and its
expected answers (file:line given per test); the oracle must reproduce them
before it is trusted as the checker of the CUDA path.
"""
import math

import numpy as np
import pytest

PI = math.pi


def _ccd_scene(bodies):
    from rigc import scene as S

    return S.Scene(bodies=bodies)


# ---------------------------------------------------------------------------
# tests/ccd/test_rigid_body_time_of_impact.cpp:170-231 ("Rigid edge-edge time
# of impact", translation section): edge A along x at height y = 1 falls to
# y_t1 onto edge B along z; toi = 1 / (1 - y_t1), impact iff y_t1 <= 0 and
# z_t0 in [-1, 1].

EE_Z = [1000.0, 10.0, 1.0 + 1e-8, 1.0, 1.0 - 1e-8, 0.5, 0.0]
EE_Y1 = [2.0, 1.0, 0.1, 1e-6, 0.0, -1e-6, -1, -2, -10, -1000]


def ee_case(z, sign, y_t1):
    from rigc import scene as S

    a = S.raw_body([[-1, 0, 0], [1, 0, 0]], edges=[[0, 1]], group_id=0)
    b = S.raw_body([[0, 0, -1], [0, 0, 1]], edges=[[0, 1]], group_id=1)
    sc = _ccd_scene([a, b])
    z_t0 = sign * z
    x0 = np.zeros(12)
    x1 = np.zeros(12)
    x0[1] = 1.0
    x0[2] = z_t0
    x1[1] = y_t1
    x1[2] = z_t0
    expected = 1 / (1 - y_t1) if y_t1 != 1 else math.inf
    hit = y_t1 <= 0.0 and -1 <= z_t0 <= 1
    return sc, x0, x1, expected, hit


@pytest.mark.parametrize("z", EE_Z)
@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("y_t1", EE_Y1)
def test_rigid_edge_edge_toi(oracle, z, sign, y_t1):
    sc, x0, x1, expected, hit = ee_case(z, sign, y_t1)
    o = oracle.OracleScene(sc)
    is_hit, toi, _ = o.edge_edge_toi(x0, x1, 0, 1, bound=1.0, tol=1e-6)
    assert is_hit == hit
    if is_hit:
        assert toi == pytest.approx(expected, abs=1e-4)  # RIGID_CCD_LENGTH_TOL
        assert toi <= expected


# tests/ccd/test_rigid_body_time_of_impact.cpp:233-303 ("Rigid face-vertex
# time of impact", translation): vertex (0, y, 1) of body B moves to z = z_t1
# against triangle (-1,0,0) (1,0,0) (0,1,0); toi = 1 / (1 - z_t1), impact iff
# z_t1 <= 0 and y in [0, 1].

FV_Y = [1.0 + 1e-8, 1.0, 1.0 - 1e-8, 0.5, 1e-8, 0.0]
FV_Z1 = [1, 1e-8, 0.0, -1e-8, -2.0, -10]


def fv_case(y, z_t1):
    from rigc import scene as S

    tri = S.raw_body([[-1, 0, 0], [1, 0, 0], [0, 1, 0]], faces=[[0, 1, 2]], group_id=0)
    pts = S.raw_body([[0, y, 1], [1, y, 1.5], [-1, y, 1.5]], faces=[[0, 1, 2]], group_id=1)
    sc = _ccd_scene([tri, pts])
    x0 = np.zeros(12)
    x1 = np.zeros(12)
    x1[6 + 2] = z_t1 - 1.0
    expected = 1 / (1 - z_t1) if z_t1 != 1 else math.inf
    hit = z_t1 <= 0.0 and 0 <= y <= 1.0
    return sc, x0, x1, expected, hit


@pytest.mark.parametrize("y", FV_Y)
@pytest.mark.parametrize("z_t1", FV_Z1)
def test_rigid_face_vertex_toi(oracle, y, z_t1):
    sc, x0, x1, expected, hit = fv_case(y, z_t1)
    o = oracle.OracleScene(sc)
    # vertex 0 of body 1 is global vertex 3; the face is face 0 of body 0
    is_hit, toi, _ = o.face_vertex_toi(x0, x1, 0, 3, bound=1.0, tol=1e-6)
    assert is_hit == hit
    if hit:
        assert toi == pytest.approx(expected, abs=1e-4)
        assert toi <= expected


# ---------------------------------------------------------------------------
# tests/interval/test_interval.cpp:12-98

def test_simple_interval_arithmetic(oracle):
    i, j = (0.0, 1.0), (4.0, 5.0)
    for op in ("add", "sub", "mul", "div"):
        lo, hi = oracle.interval_op(op, i, j)
        assert lo <= hi
    lo, hi = oracle.interval_op("div", (1.0, 1.0), j)
    assert lo <= hi
    lo, hi = oracle.interval_op("add", i, (10.0, 10.0))
    assert lo == pytest.approx(10, abs=1e-12) and hi == pytest.approx(11, abs=1e-12)


@pytest.mark.parametrize("shift", [0, 2 * PI, -2 * PI, 100 * PI, -100 * PI])
def test_cosine_interval(oracle, shift):
    def icos(a, b):
        x = oracle.interval_op("add", (a, b), (shift, shift))
        return oracle.interval_op("cos", x)

    r = icos(-1, 7)
    assert r == (-1.0, 1.0)
    assert icos(2, 4)[1] < 0
    assert icos(0, 1)[0] > 0
    r = icos(1, 2)
    assert r[0] < 0 < r[1]


@pytest.mark.parametrize("shift", [0, 2 * PI, -2 * PI, 100 * PI, -100 * PI])
def test_sine_interval(oracle, shift):
    shift = shift + PI / 2

    def isin(a, b):
        x = oracle.interval_op("add", (a, b), (shift, shift))
        return oracle.interval_op("sin", x)

    assert isin(-1, 7) == (-1.0, 1.0)
    assert isin(2, 4)[1] < 0
    assert isin(0, 1)[0] > 0
    r = isin(1, 2)
    assert r[0] < 0 < r[1]


# tests/utils/test_sinc.cpp:14-110

@pytest.mark.parametrize("x,expected", [
    ((0.0, 0.0), (1.0, 1.0)), ((0.0, 1e-8), (1.0, 1.0)), ((-1e-8, 0.0), (1.0, 1.0)),
    ((-1e-8, 1e-8), (1.0, 1.0)),
    ((0.0, PI), (0.0, 1.0)), ((-PI, 0.0), (0.0, 1.0)), ((-PI, PI), (0.0, 1.0)),
    ((0.0, PI / 2), (2 / PI, 1.0)), ((-PI / 2, 0.0), (2 / PI, 1.0)),
    ((-PI / 2, PI / 2), (2 / PI, 1.0)),
])
def test_interval_sinc(oracle, x, expected):
    lo, hi = oracle.interval_op("sinc", x)
    assert lo == pytest.approx(expected[0], abs=1e-8)
    assert hi == pytest.approx(expected[1], abs=1e-8)


def _sinc(x):
    return 1.0 if x == 0 else math.sin(x) / x


@pytest.mark.parametrize("x,expected", [
    ((-5, 5), (-0.217233628211, 1)), ((-1, 5), (-0.217233628211, 1)),
    ((0, 5), (-0.217233628211, 1)), ((5, 7), (_sinc(5), _sinc(7))),
    ((21, 22), (_sinc(22), _sinc(21))),
])
def test_interval_sinc_looser_bounds(oracle, x, expected):
    lo, hi = oracle.interval_op("sinc", (float(x[0]), float(x[1])))
    assert lo <= expected[0] and expected[1] <= hi          # subset(expected, y)
    assert -0.23 <= lo and hi <= 1                           # subset(y, [-0.23, 1])
    if x[0] > 0:
        assert -1 / x[0] <= lo and hi <= 1 / x[0]


# tests/physics/test_pose.cpp:42-66: rotation vector -> matrix vs angle-axis

def test_rotation_matrix_angle_axis(oracle):
    rng = np.random.default_rng(0)
    for k in range(101):
        angle = 0.0 if k == 0 else rng.uniform(0, 2 * PI)
        axis = rng.uniform(-1, 1, 3)
        axis /= np.linalg.norm(axis)
        R = oracle.rotation_matrix(angle * axis)
        K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
        Rexp = np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * K @ K
        assert np.linalg.norm(R - Rexp) < 1e-12


# tests/barrier/test_barriers.cpp:9-49: barrier gradient / Hessian by finite
# differences for s = 10^[-5, 1]

@pytest.mark.parametrize("s_exp", [-5, -3, -1, 0, 1])
def test_ipc_barrier_finite_differences(oracle, s_exp):
    s = 10.0 ** s_exp
    for frac in (0.05, 0.3, 0.7, 0.95):
        d = frac * s
        h = 1e-7 * s
        b0 = oracle.barrier(d, s)
        bp, bm = oracle.barrier(d + h, s), oracle.barrier(d - h, s)
        g_fd = (bp - bm) / (2 * h)
        def grad(d):
            return (s - d) * (2 * math.log(d / s) - s / d + 1)

        assert grad(d) == pytest.approx(g_fd, rel=1e-5, abs=1e-12 * max(1, abs(b0)))
        hess_fd = (grad(d + h) - grad(d - h)) / (2 * h)
        hess = (s / d + 2) * s / d - 2 * math.log(d / s) - 3
        assert hess == pytest.approx(hess_fd, rel=1e-5)
    assert oracle.barrier(s, s) == 0.0 and oracle.barrier(2 * s, s) == 0.0
    assert math.isinf(oracle.barrier(0.0, s))


# ---------------------------------------------------------------------------
# derivative checks of the oracle's own autodiff (the reference checks its
# energy and barrier derivatives by finite differences the same way,
# src/problems/distance_barrier_rb_problem.cpp:819-841, 1385-1396)

def test_body_energy_finite_differences(oracle, cube_scene):
    sc = cube_scene
    body = sc.bodies[4]
    rng = np.random.default_rng(2)
    x = body.pose + rng.normal(0, 0.2, 6)
    e, g, H = oracle.body_energy(body, x, sc.gravity, sc.timestep)
    h = 1e-6
    for i in range(6):
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        ep, gp, _ = oracle.body_energy(body, xp, sc.gravity, sc.timestep)
        em, gm, _ = oracle.body_energy(body, xm, sc.gravity, sc.timestep)
        assert g[i] == pytest.approx((ep - em) / (2 * h), rel=1e-6, abs=1e-6)
        assert np.allclose(H[:, i], (gp - gm) / (2 * h), rtol=1e-5, atol=1e-5)


def test_barrier_local_terms_finite_differences(oracle, cube_scene):
    from conftest import contact_poses

    sc = cube_scene
    x = contact_poses(sc)
    o = oracle.OracleScene(sc)
    ee, fv = o.detect_candidates(x, continuous=False, inflation=5e-4)
    cs = o.constraint_set(x, ee, fv, 1e-3)
    assert len(cs) > 0
    e, g, H = o.local_terms(x, cs, 1e-3, project=False)
    h = 1e-7
    for ci in range(min(len(cs), 6)):
        one = oracle.Constraints(cs.types[ci:ci + 1], cs.verts[ci:ci + 1], cs.prims[ci:ci + 1],
                                 cs.bodies[ci:ci + 1], cs.weight[ci:ci + 1], cs.eps[ci:ci + 1])
        b0, b1 = cs.bodies[ci]
        for k in range(12):
            dof = 6 * (b0 if k < 6 else b1) + k % 6
            xp, xm = x.copy(), x.copy()
            xp[dof] += h
            xm[dof] -= h
            ep, gp, _ = o.local_terms(xp, one, 1e-3, project=False)
            em, gm, _ = o.local_terms(xm, one, 1e-3, project=False)
            assert g[ci][k] == pytest.approx((ep[0] - em[0]) / (2 * h), rel=1e-4,
                                             abs=1e-6 * np.abs(g[ci]).max())
            col = (gp[0] - gm[0]) / (2 * h)
            assert np.allclose(H[ci][:, k], col, rtol=1e-4, atol=1e-5 * np.abs(H[ci]).max())


def test_psd_projection_matches_eigh(oracle):
    rng = np.random.default_rng(0)
    for _ in range(20):
        A = rng.normal(size=(12, 12))
        A = A + A.T
        P = oracle.project_to_psd(A)
        w, V = np.linalg.eigh(A)
        ref = (V * np.maximum(w, 0)) @ V.T
        assert np.abs(P - ref).max() <= 1e-10 * np.abs(ref).max()
    S = rng.normal(size=(12, 12))
    S = S @ S.T + np.eye(12)
    assert np.array_equal(oracle.project_to_psd(S), S)   # PSD input returned unchanged


def test_hash_grid_equals_brute_force(oracle, cube_scene):
    from conftest import contact_poses

    sc = cube_scene
    x0 = contact_poses(sc)
    x1 = sc.predictor_poses(x0)
    o = oracle.OracleScene(sc)
    for cont, infl in ((True, 0.0), (False, 5e-4), (False, 1e-2)):
        a = o.detect_candidates(x0, x1, cont, infl)
        b = o.detect_candidates(x0, x1, cont, infl, brute=True)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_hash_grid_equals_brute_force_on_a_pile(oracle):
    """The same on an icosphere contact pile (thousands of grid items, so
    the threads' chunks of items, sorts and cell runs all meet boundaries)."""
    import bench

    sc, x0, x1 = bench.make_workload(8, 0)
    o = oracle.OracleScene(sc)
    for cont, infl in ((True, 0.0), (False, 5e-4)):
        a = o.detect_candidates(x0, x1, cont, infl)
        b = o.detect_candidates(x0, x1, cont, infl, brute=True)
        assert len(a[0]) + len(a[1]) > 0
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def parallel_edges(offset, direction=(1.0, 2e-5, 1e-5)):
    """Two single-edge bodies whose edges are nearly parallel (mollified) and
    whose closest features are endpoints for the given offset of the second."""
    from rigc import scene as S

    a = S.raw_body([[0, 0, 0], [1, 0, 0]], edges=[[0, 1]], group_id=0)
    b = S.raw_body(np.array([[0, 0, 0], direction]) + np.asarray(offset), edges=[[0, 1]],
                   group_id=1)
    return S.Scene(bodies=[a, b])


PARALLEL_CASES = {"point-point": [1.0004, 3e-4, 0.0], "point-edge": [0.6, 4e-4, 1e-4]}


@pytest.mark.parametrize("case", sorted(PARALLEL_CASES))
def test_mollified_ee_endpoint_distance(oracle, case):
    """Near-parallel EE pairs whose closest points are endpoints stay EE
    constraints (mollified); their barrier uses the closest-feature distance,
    so the energy is continuous as the pair enters the set and its
    derivatives match finite differences."""
    sc = parallel_edges(PARALLEL_CASES[case])
    o = oracle.OracleScene(sc)
    x = np.zeros(12)
    x[9:12] = [1e-6, -2e-6, 1.5e-6]
    ee, fv = o.detect_candidates(x, continuous=False, inflation=5e-4)
    cs = o.constraint_set(x, ee, fv, 1e-3)
    assert list(cs.types) == [2]
    e, g, H = o.local_terms(x, cs, 1e-3, project=False)
    h = 1e-7
    for k in range(12):
        xp, xm = x.copy(), x.copy()
        xp[k] += h
        xm[k] -= h
        ep, gp, _ = o.local_terms(xp, cs, 1e-3, project=False)
        em, gm, _ = o.local_terms(xm, cs, 1e-3, project=False)
        assert g[0][k] == pytest.approx((ep[0] - em[0]) / (2 * h), rel=1e-4,
                                        abs=1e-5 * np.abs(g[0]).max())
        assert np.allclose(H[0][:, k], (gp[0] - gm[0]) / (2 * h), rtol=1e-4,
                           atol=1e-5 * np.abs(H[0]).max())
    # moving the pair apart to the activation distance takes the energy to 0
    # smoothly: no jump where the segment distance crosses dhat
    es = []
    for t in np.linspace(0.0, 1.0, 41):
        xt = x.copy()
        xt[7] = t * 1e-3
        ee, fv = o.detect_candidates(xt, continuous=False, inflation=5e-4)
        cs_t = o.constraint_set(xt, ee, fv, 1e-3)
        es.append(o.local_terms(xt, cs_t, 1e-3)[0].sum() if len(cs_t) else 0.0)
    es = np.array(es)
    assert es[-1] == 0.0 and np.all(np.diff(es) <= 1e-30)
