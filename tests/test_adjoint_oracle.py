"""Adjoint of the time step on the CPU oracle: implicit differentiation of
each converged step, checked against central finite differences (h = 1e-6)
of the oracle's own simulator on a small contact scene.

Scene: two unit cubes just above a static plane, falling at 1 m/s, the second
sliding toward the first, so the steps see cube-plane and cube-cube contacts.
Loss: the squared distance of cube 0's final centre to (3, 0, 0.5).  The
parameters are the cubes' initial linear and angular velocities (omega in
body coordinates, Qdot0 = R(theta0) [omega]x)."""

import numpy as np
import pytest

H = 0.01
G = (0.0, -9.81, 0.0)
DHAT = 1e-3
TARGET = np.array([3.0, 0.0, 0.5])
STEPS = 4
# differentiable settings: tight convergence, Newton polish, CCD step rescaling
DIFF = dict(velocity_conv_tol=1e-10, velocity_conv_tol_abs=1, newton_polish=8, ccd_rescale=0.8)
FD_H = 1e-6
FD_RTOL = 1e-5


def contact_pair_spec(seed=3):
    from rigc import meshes, scene as S

    rng = np.random.default_rng(seed)
    spec = S._base_spec(H, DHAT, STEPS)
    V, F = meshes.cube()
    bodies = spec["rigid_body_problem"]["rigid_bodies"]
    for pos, vel in (([0.0, 0.515, 0.0], [0.0, -1.0, 0.0]),
                     ([1.008, 0.52, 0.0], [-0.6, -1.0, 0.05])):
        R = S.lattice_rotation(rng, max_deg=0.2)
        bodies.append(S._rb(V, F, position=pos, rotation=S.matrix_to_euler_xyz_deg(R).tolist(),
                            linear_velocity=vel,
                            angular_velocity=rng.normal(0, 20.0, 3).tolist()))
    Vp, Fp = meshes.plane(20.0)
    bodies.append(S._rb(Vp, Fp, position=[0, 0, 0], is_dof_fixed=True, type="static"))
    return spec


def contact_pair():
    from rigc import scene as S

    return S.scene_from_json(contact_pair_spec())


def qdot_of(poses, omega):
    from rigc import scene as S

    return np.stack([S.rotvec_to_matrix(p[3:6]) @ S.hat(w) for p, w in zip(poses, omega)]
                    ).reshape(-1)


def oracle_rollout(oracle, sc, dvel=None, record=False, steps=STEPS):
    """Oracle rollout from the scene's state with the velocities (v, omega)
    perturbed by dvel (nb x 6); returns (loss, sim)."""
    sim = oracle.OracleSim(sc, h=H, gravity=G, dhat=DHAT, **DIFF)
    nb = len(sim.mass)
    poses = sim.pose.reshape(nb, 6)
    vel = sim.vel.reshape(nb, 6).copy()
    if dvel is not None:
        vel = vel + dvel
    sim.vel = np.ascontiguousarray(vel.reshape(-1))
    sim.Qdot = np.ascontiguousarray(qdot_of(poses, vel[:, 3:]))
    sim.rollout(steps, record=record)
    c = sim.pose.reshape(nb, 6)[0, :3]
    return float(((c - TARGET) ** 2).sum()), sim


def omega_gradient(poses, gQ):
    """dL/domega from dL/dQdot0 with Qdot0 = R(theta0) [omega]x."""
    from rigc import scene as S

    out = np.zeros((len(poses), 3))
    for b, p in enumerate(poses):
        R = S.rotvec_to_matrix(p[3:6])
        for j in range(3):
            e = np.zeros(3)
            e[j] = 1
            out[b, j] = (gQ[b].reshape(3, 3) * (R @ S.hat(e))).sum()
    return out


def oracle_gradient(oracle, sc, steps=STEPS):
    """(loss, dL/d(v, omega) nb x 6, sim) by the oracle's adjoint."""
    L, sim = oracle_rollout(oracle, sc, record=True, steps=steps)
    nb = len(sim.mass)
    dp = np.zeros((nb, 6))
    dp[0, :3] = 2 * (sim.pose.reshape(nb, 6)[0, :3] - TARGET)
    gp, gv, gq = sim.backward(dp)
    poses0 = sc.poses().reshape(nb, 6)
    return L, np.concatenate([gv[:, :3], omega_gradient(poses0, gq)], 1), sim


def fd_directional(oracle, sc, d, h=FD_H, steps=STEPS):
    Lp, _ = oracle_rollout(oracle, sc, d * h, steps=steps)
    Lm, _ = oracle_rollout(oracle, sc, -d * h, steps=steps)
    return (Lp - Lm) / (2 * h)


def fd_directions(nb, dynamic, k=2, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(k):
        d = rng.normal(size=(nb, 6))
        d[~dynamic] = 0
        out.append(d)
    return out


@pytest.fixture(scope="module")
def pair_gradient(oracle):
    sc = contact_pair()
    L, g, sim = oracle_gradient(oracle, sc)
    return sc, L, g, sim


def test_scene_has_contacts(oracle, pair_gradient):
    sc, L, g, sim = pair_gradient
    o = oracle.OracleScene(sc)
    pairs = set()
    for _, x, _ in sim.tape:
        ee, fv = o.detect_candidates(x, continuous=False, inflation=DHAT / 2)
        cs = o.constraint_set(x, ee, fv, DHAT)
        pairs |= {tuple(sorted(map(int, b))) for b in cs.bodies}
    assert len(sim.tape) == STEPS
    assert np.isfinite(L) and np.all(np.isfinite(g))
    plane = sc.num_bodies - 1
    assert (0, 1) in pairs and any(plane in p for p in pairs)


def test_adjoint_matches_central_differences(oracle, pair_gradient):
    sc, L, g, sim = pair_gradient
    nb = sc.num_bodies
    dyn = np.array([b.type == 2 for b in sc.bodies])
    for d in fd_directions(nb, dyn):
        ad = float((g * d).sum())
        fd = fd_directional(oracle, sc, d)
        assert abs(ad - fd) <= FD_RTOL * abs(fd), (ad, fd)


def test_adjoint_free_fall_closed_form(oracle):
    """Far from contact: p_T = p_0 + T h v_0 + h^2 g T(T+1)/2, so
    dL/dv_0 = 2 (p_T - target) T h."""
    from rigc import meshes, scene as S

    V, F = meshes.cube()
    sc = S.Scene(bodies=[S.make_body(V, F, position=(0, 5, 0), linear_velocity=(0.3, 1.0, -0.2))])
    T = 5
    L, g, sim = oracle_gradient(oracle, sc, steps=T)
    pT = sim.pose[:3]
    assert np.allclose(g[0, :3], 2 * (pT - TARGET) * T * H, rtol=1e-12, atol=1e-14)
    assert np.abs(g[0, 3:]).max() <= 1e-12


def test_lattice_adjoint_matches_differences_of_every_parameter():
    """The differentiation workload's stored gradient (the oracle's adjoint
    over the 64 cubes' 384 initial linear and angular velocities, 50 steps,
    tests/golden/adjoint_cube_lattice.npz) against central differences of the
    oracle's simulator in every one of the 384 parameters at h = 1e-6 and
    h / 2 (tests/golden/adjoint_cube_lattice_fd.npz, made by
    make_adjoint_fixture.py --all-parameters): the differences converge at
    second order (the h / 2 error a quarter of the h one) and their
    extrapolation (4 D(h/2) - D(h)) / 3 meets the adjoint to 1e-7 of the
    largest component."""
    import os

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    g = np.load(os.path.join(here, "adjoint_cube_lattice.npz"))["grad"][:64]
    fd = np.load(os.path.join(here, "adjoint_cube_lattice_fd.npz"))
    assert fd["fd_h"].shape == (64, 6) and float(fd["h"]) == 1e-6
    scale = np.abs(fd["fd_extrapolated"]).max()
    err_h = np.abs(g - fd["fd_h"]).max()
    err_h2 = np.abs(g - fd["fd_h2"]).max()
    assert err_h2 < 0.5 * err_h  # second order: ~1/4
    assert err_h <= 1e-5 * scale
    assert np.abs(g - fd["fd_extrapolated"]).max() <= 1e-7 * scale
