"""The oracle's piecewise-linear CCD (trajectory PIECEWISE_LINEAR,
src/ccd/piecewise_linear/time_of_impact.cpp) on analytic cases and on the
reference's own CCD queries, checked the way the reference's tests check it
(tests/ccd/test_rigid_body_time_of_impact.cpp:597-853):

* wrecking-ball and ccd-test queries ("Failing earliest tois"): when the
  piecewise-linear CCD reports an impact at toi, the rigid CCD from t0 to the
  poses at toi finds none;
* kinematic queries ("toi=0"): an impact is reported at toi > 0, and for
  edge-edge queries the squared distance of the edges at toi is 0 to 1e-10.
"""
import numpy as np
import pytest

from test_reference_fixtures import queries


def two_body_scene(VA, EA, FA, VB, EB, FB):
    """Two raw bodies (rest vertices as given); edges from the faces when
    faces are given."""
    from rigc import scene as S

    def body(V, E, F, g):
        if F is not None:
            return S.raw_body(np.asarray(V, float), faces=np.asarray(F, np.int32), group_id=g)
        return S.raw_body(np.asarray(V, float), edges=np.asarray(E, np.int32).reshape(-1, 2), group_id=g)

    return S.Scene(bodies=[body(VA, EA, FA, 0), body(VB, EB, FB, 1)])


def edge_pair(drop=2.0, spin=0.0):
    """Edge A on the x axis; edge B along z at height 1 falling by `drop` (and
    turning by `spin` radians about y) over the step."""
    sc = two_body_scene([[-1, 0, 0], [1, 0, 0]], [[0, 1]], None,
                        [[0, 1, -1], [0, 1, 1]], [[0, 1]], None)
    x0 = np.zeros(12)
    x1 = np.zeros(12)
    x1[7] = -drop
    x1[10] = spin
    return sc, x0, x1


@pytest.mark.parametrize("ms", [0.0, 1e-6, 1e-4, 1e-3, 0.1])
def test_linear_ccd_translating_edges(oracle, ms):
    """The linear CCD alone: edge B falls onto edge A at speed 2 from height
    1; the first time the gap 1 - 2 t reaches ms, within the co-domain
    tolerance (1e-6 + ms of the gap) and never after it, in a few hundred
    boxes."""
    p0 = [[-1, 0, 0], [1, 0, 0], [0, 1, -1], [0, 1, 1]]
    p1 = [[-1, 0, 0], [1, 0, 0], [0, -1, -1], [0, -1, 1]]
    hit, toi, boxes, status = oracle.linear_ccd(p0, p1, ms)
    exact = (1.0 - ms) / 2.0
    assert hit and status == 0 and boxes < 1000
    assert exact - (1e-6 + ms) <= toi <= exact


def test_linear_ccd_vertex_and_triangle(oracle):
    """A vertex falling onto a triangle at t = 0.25, and beside it (no impact:
    u + v > 1 there)."""
    tri = [[-1, 0, -1], [1, 0, -1], [0, 0, 1]]
    hit, toi, _, _ = oracle.linear_ccd([[0, 0.5, 0]] + tri, [[0, -1.5, 0]] + tri, fv=True)
    assert hit and 0.25 - 1e-6 <= toi <= 0.25
    hit, toi, _, _ = oracle.linear_ccd([[0.9, 0.5, 0.9]] + tri, [[0.9, -1.5, 0.9]] + tri, fv=True)
    assert not hit


def test_linear_ccd_parallel_edges(oracle):
    """Parallel edges sliding past at a gap of 2e-6 with ms = 1e-6: boxes
    along the whole overlap stay near the separation, the search ends within
    its budget either way, and an impact, if reported, comes from the
    co-domain tolerance (it is conservative)."""
    p0 = [[0, 0, 0], [1, 0, 0], [0.5, 2e-6, 0], [1.5, 2e-6, 0]]
    p1 = [[0, 0, 0], [1, 0, 0], [-0.5, 2e-6, 0], [0.5, 2e-6, 0]]
    hit, toi, boxes, status = oracle.linear_ccd(p0, p1, 1e-6)
    assert boxes <= 1000000 and status in (0, 5)


def test_translating_edges(oracle):
    """The piecewise-linear CCD of a falling edge: the interval bound of a
    piece's deviation from the straight line holds the whole displacement
    (the reference's interval expression), so pieces are halved until it is
    below half the gap, and the impact is reported at the start of the first
    piece whose gap fell below 0.2 of the initial one (the reference's
    decreasing-distance rule): never after the exact contact time."""
    sc, x0, x1 = edge_pair()
    o = oracle.OracleScene(sc)
    for dmin in (0.0, 1e-3, 0.1):
        hit, toi, st = o.pl_toi(x0, x1, 0, 0, 1, dmin=dmin)
        assert hit and st["status"] == 0 and st["pieces"] > 1
        assert 0 < toi <= (1.0 - dmin) / 2.0
        assert 1 - 2 * toi < 0.2  # the gap at toi


def test_separating_edges_miss(oracle):
    sc, x0, x1 = edge_pair(drop=-1.0)
    o = oracle.OracleScene(sc)
    hit, toi, _ = o.pl_toi(x0, x1, 0, 0, 1)
    assert not hit and np.isinf(toi)


def test_vertex_onto_triangle(oracle):
    """A vertex falling onto a triangle (FV) lands at t = 0.25."""
    sc = two_body_scene([[-1, 0, -1], [1, 0, -1], [0, 0, 1]], [[0, 1], [1, 2], [2, 0]],
                        [[0, 1, 2]], [[0, 0.5, 0]], np.zeros((0, 2)), None)
    x0 = np.zeros(12)
    x1 = np.zeros(12)
    x1[7] = -2.0
    o = oracle.OracleScene(sc)
    hit, toi, st = o.pl_toi(x0, x1, 1, 0, 3)
    assert hit and 0 < toi <= 0.25
    # beside the triangle: no impact
    x1[6] = 5.0
    hit, toi, _ = o.pl_toi(x0, x1, 1, 0, 3)
    assert not hit


def test_rotating_edge_is_conservative(oracle):
    """A falling and turning edge: the impact is not after the rigid
    trajectory's own (the rigid CCD up to it finds none)."""
    sc, x0, x1 = edge_pair(drop=2.0, spin=3.0)
    o = oracle.OracleScene(sc)
    hit, toi, st = o.pl_toi(x0, x1, 0, 0, 1)
    assert hit and st["pieces"] > 1 and 0 < toi <= 0.5
    xt = (x1 - x0) * toi + x0
    h2, _, _ = o.edge_edge_toi(x0, xt, 0, 1)
    assert not h2
    rig, t_rigid, _ = o.edge_edge_toi(x0, x1, 0, 1)
    assert rig and toi <= t_rigid


def _segment_sqdist(a0, a1, b0, b1):
    """Squared distance of two segments (closest points by clamped
    parameters; a check only)."""
    d1, d2, r = a1 - a0, b1 - b0, a0 - b0
    a, e, f = d1 @ d1, d2 @ d2, d2 @ r
    c, b = d1 @ r, d1 @ d2
    den = a * e - b * b
    s = np.clip((b * f - c * e) / den, 0, 1) if den > 1e-300 else 0.0
    t = (b * s + f) / e
    if t < 0:
        t, s = 0.0, np.clip(-c / a, 0, 1)
    elif t > 1:
        t, s = 1.0, np.clip((b - c) / a, 0, 1)
    d = (a0 + d1 * s) - (b0 + d2 * t)
    return float(d @ d)


@pytest.fixture(scope="module")
def pl_queries(oracle):
    import make_reference_fixtures as M

    q = queries()
    out = []
    for k, V, P, name in zip(q["kind"], q["vertices"], q["poses"], q["name"]):
        sc = M.query_scene(int(k), V)
        o = oracle.OracleScene(sc)
        x0 = np.concatenate([P[0, 0], P[1, 0]])
        x1 = np.concatenate([P[0, 1], P[1, 1]])
        hit, toi, st = o.pl_toi(x0, x1, int(k), 0, 1 if k == 0 else 3)
        out.append((str(name), int(k), sc, o, x0, x1, hit, toi, st))
    return out


def test_reference_queries_conservative(pl_queries):
    """"Failing earliest tois": no rigid impact before the piecewise-linear one."""
    checked = 0
    for name, k, sc, o, x0, x1, hit, toi, st in pl_queries:
        if "kinematic" in name or not hit:
            continue
        xt = (x1 - x0) * toi + x0
        h2 = (o.edge_edge_toi(x0, xt, 0, 1) if k == 0 else o.face_vertex_toi(x0, xt, 0, 3))[0]
        assert not h2, name
        checked += 1
    assert checked > 50


def test_reference_kinematic_queries(pl_queries):
    """"toi=0": the queries whose bodies start in contact get toi > 0, and the
    edges are in contact (squared distance <= 1e-10) at it."""
    seen = 0
    for name, k, sc, o, x0, x1, hit, toi, st in pl_queries:
        if "kinematic" not in name:
            continue
        seen += 1
        assert hit and toi > 0, name
        if k == 0:
            V = sc.world_vertices((x1 - x0) * toi + x0)
            assert _segment_sqdist(V[0], V[1], V[2], V[3]) <= 1e-10, name
    assert seen == 13


def test_earliest_over_candidates(oracle, pl_queries):
    """pl_earliest_toi is the smallest per-candidate time, threads or not."""
    name, k, sc, o, x0, x1, hit, toi, st = next(q for q in pl_queries if q[6] and q[1] == 0)
    t, per, stats = o.pl_earliest_toi(x0, x1, [[0, 1]], np.zeros((0, 2)), nthreads=2)
    assert t == toi and per[0] == toi and stats["boxes"] == st["boxes"]
