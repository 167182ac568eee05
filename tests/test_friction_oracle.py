"""Friction oracle checks on the CPU: a known answer, finite differences of
the gradient and Hessian, and invariance under the choice of tangent basis.

The reference computes lagged friction with ipc-toolkit
(construct_friction_constraint_set, compute_potential / _gradient / _hessian
as called in src/problems/distance_barrier_rb_problem.cpp:168-188,
1411-1572); its test suite has no friction fixtures, so the oracle is pinned
here by the IPC friction formulation itself (Li et al. 2020, sec. 5).
"""
import numpy as np
import pytest

DHAT = 1e-3
KAPPA = 1e4
MU = 0.5
EPSVH = 1e-3 * 1e-2  # static_friction_speed_bound * timestep


def _barrier_d1(d, s):
    return (s - d) * (2 * np.log(d / s) - s / d + 1)


def point_on_triangle(gap):
    """A static triangle in the z = 0 plane and a body whose first vertex
    hovers gap above the triangle's interior (its other vertices are far)."""
    from rigc import scene as S

    tri = S.raw_body([[-1, 0, 0], [1, 0, 0], [0, 1, 0]], faces=[[0, 1, 2]], group_id=0,
                     body_type="static")
    pts = S.raw_body([[0, 0.3, gap], [1, 0.3, 1.5], [-1, 0.3, 1.5]], faces=[[0, 1, 2]],
                     group_id=1)
    return S.Scene(bodies=[tri, pts])


def _constraints(o, x0):
    ee, fv = o.detect_candidates(x0, continuous=False, inflation=DHAT / 2)
    return o.constraint_set(x0, ee, fv, DHAT)


@pytest.mark.parametrize("slide", [3e-4, 2e-6])
def test_friction_known_answer(oracle, slide):
    gap = 4e-4
    sc = point_on_triangle(gap)
    o = oracle.OracleScene(sc)
    x0 = np.zeros(12)
    cs = _constraints(o, x0)
    fv = [i for i in range(len(cs)) if cs.types[i] == 3]
    assert len(fv) == 1
    lam, params, T = o.friction_constraints(x0, cs, DHAT, KAPPA)
    i = fv[0]
    expect_lam = -KAPPA * _barrier_d1(gap * gap, DHAT * DHAT) * 2 * gap
    assert lam[i] == pytest.approx(expect_lam, rel=1e-12)
    # closest point of (0, 0.3) in the triangle's barycentric frame
    assert params[i] == pytest.approx([0.35, 0.3], abs=1e-14)
    # the basis spans the triangle's plane
    assert np.abs(T[i][:, 2]).max() < 1e-15
    assert np.allclose(T[i] @ T[i].T, np.eye(2), atol=1e-15)
    # slide the point body along x
    x = x0.copy()
    x[6] = slide
    e, g, H = o.friction_local_terms(x, x0, cs, (lam, params, T), MU, EPSVH, project=False)
    if slide >= EPSVH:
        f0 = slide
    else:
        f0 = -slide ** 3 / (3 * EPSVH ** 2) + slide ** 2 / EPSVH + EPSVH / 3
    assert e[i] == pytest.approx(MU * lam[i] * f0, rel=1e-12)
    # the friction force opposes the slide: the energy grows with the point
    # body's x (local body 0 of a face-vertex constraint is the vertex's)
    assert g[i][0] > 0 and abs(g[i][1]) < 1e-12 * g[i][0]
    assert g[i][6] == pytest.approx(-g[i][0], rel=1e-12)


def _friction_setup(oracle, cube_scene, cube_contact, seed):
    o = oracle.OracleScene(cube_scene)
    x0 = cube_contact
    cs = _constraints(o, x0)
    assert len(cs) > 0
    fc = o.friction_constraints(x0, cs, DHAT, KAPPA)
    rng = np.random.default_rng(seed)
    nb = cube_scene.num_bodies
    dyn = np.array([b.type == 2 for b in cube_scene.bodies])
    dx = np.zeros((nb, 6))
    dx[:, [0, 2]] = rng.normal(0, 3e-4, (nb, 2))
    dx[:, 3:] = rng.normal(0, 2e-4, (nb, 3))
    dx[~dyn] = 0
    return o, x0, cs, fc, x0 + dx.reshape(-1)


def test_friction_gradient_fd(oracle, cube_scene, cube_contact):
    o, x0, cs, fc, x = _friction_setup(oracle, cube_scene, cube_contact, 1)
    e, g, _ = o.friction_term(x, x0, cs, fc, MU, EPSVH, project=False)
    assert e > 0
    h = 1e-8
    active = np.flatnonzero(np.abs(g) > 0)
    assert len(active) > 0
    for k in active[:24]:
        xp, xm = x.copy(), x.copy()
        xp[k] += h
        xm[k] -= h
        ep = o.friction_term(xp, x0, cs, fc, MU, EPSVH, project=False)[0]
        em = o.friction_term(xm, x0, cs, fc, MU, EPSVH, project=False)[0]
        fd = (ep - em) / (2 * h)
        assert fd == pytest.approx(g[k], rel=1e-5, abs=1e-7 * np.abs(g).max())


def test_friction_hessian_fd(oracle, cube_scene, cube_contact):
    o, x0, cs, fc, x = _friction_setup(oracle, cube_scene, cube_contact, 2)
    _, g, (rp, col, val) = o.friction_term(x, x0, cs, fc, MU, EPSVH, project=False)
    nb = cube_scene.num_bodies
    Hd = np.zeros((6 * nb, 6 * nb))
    for r in range(nb):
        for k in range(rp[r], rp[r + 1]):
            Hd[6 * r:6 * r + 6, 6 * col[k]:6 * col[k] + 6] = val[k]
    assert np.allclose(Hd, Hd.T, rtol=0, atol=1e-9 * np.abs(Hd).max())
    h = 1e-8
    active = np.flatnonzero(np.abs(g) > 0)
    for k in active[:12]:
        xp, xm = x.copy(), x.copy()
        xp[k] += h
        xm[k] -= h
        gp = o.friction_term(xp, x0, cs, fc, MU, EPSVH, project=False)[1]
        gm = o.friction_term(xm, x0, cs, fc, MU, EPSVH, project=False)[1]
        fd = (gp - gm) / (2 * h)
        scale = np.abs(Hd[:, k]).max()
        assert np.abs(fd - Hd[:, k]).max() <= 1e-4 * scale + 1e-9


def test_friction_basis_invariance(oracle, cube_scene, cube_contact):
    """Any orthonormal basis of the tangent plane gives the same potential."""
    o, x0, cs, fc, x = _friction_setup(oracle, cube_scene, cube_contact, 3)
    lam, params, T = fc
    rng = np.random.default_rng(4)
    phi = rng.uniform(0, 2 * np.pi, len(cs))
    c, s = np.cos(phi), np.sin(phi)
    T2 = np.empty_like(T)
    T2[:, 0] = c[:, None] * T[:, 0] + s[:, None] * T[:, 1]
    T2[:, 1] = -(-s[:, None] * T[:, 0] + c[:, None] * T[:, 1])  # flipped orientation
    e1, g1, H1 = o.friction_local_terms(x, x0, cs, fc, MU, EPSVH)
    e2, g2, H2 = o.friction_local_terms(x, x0, cs, (lam, params, T2), MU, EPSVH)
    assert np.allclose(e1, e2, rtol=1e-12, atol=0)
    assert np.allclose(g1, g2, rtol=1e-10, atol=1e-12 * np.abs(g1).max())
    assert np.allclose(H1, H2, rtol=1e-9, atol=1e-10 * np.abs(H1).max())


def test_friction_psd(oracle, cube_scene, cube_contact):
    o, x0, cs, fc, x = _friction_setup(oracle, cube_scene, cube_contact, 5)
    _, _, H = o.friction_local_terms(x, x0, cs, fc, MU, EPSVH, project=True)
    for Hi in H:
        w = np.linalg.eigvalsh(0.5 * (Hi + Hi.T))
        assert w.min() >= -1e-10 * max(abs(w).max(), 1e-300)
