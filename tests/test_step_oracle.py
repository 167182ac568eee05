"""The oracle's restated time step (DistanceBarrierRBProblem::simulation_step
with the IPC Newton solver) on the CPU: a closed-form free fall, and a few
steps of the 27-cube scene staying intersection-free."""
import numpy as np
import pytest

H = 0.01
G = (0.0, -9.81, 0.0)


def free_cube():
    from rigc import meshes, scene as S

    V, F = meshes.cube()
    b = S.make_body(V, F, position=(0, 5, 0), linear_velocity=(0.3, 1.0, -0.2))
    return S.Scene(bodies=[b])


def test_free_fall_closed_form(oracle):
    """Far from everything, implicit Euler: v1 = v0 + h g, p1 = p0 + h v1."""
    sc = free_cube()
    sim = oracle.OracleSim(sc, h=H, gravity=G, dhat=1e-3)
    p = sc.poses()[:3].copy()
    v = sc.velocities()[:3].copy()
    for _ in range(3):
        sim.step()
        v = v + H * np.array(G)
        p = p + H * v
        assert np.allclose(sim.pose[:3], p, rtol=0, atol=1e-12)
        assert np.allclose(sim.vel[:3], v, rtol=0, atol=1e-10)
    # the rotation does not move (zero angular velocity)
    assert np.allclose(sim.pose[3:], sc.poses()[3:], atol=1e-14)


def test_cube_lattice_steps(oracle, cube_scene):
    sim = oracle.OracleSim(cube_scene, h=H, gravity=G, dhat=1e-3)
    o = oracle.OracleScene(cube_scene)
    y0 = sim.pose.reshape(-1, 6)[:, 1].copy()
    for _ in range(3):
        st = sim.step()
        assert st[0] >= 1
        # no intersection: every constraint distance stays positive
        x = sim.pose
        ee, fv = o.detect_candidates(x, continuous=False, inflation=5e-4)
        cs = o.constraint_set(x, ee, fv, 1e-3)
        e, _, _ = o.local_terms(x, cs, 1e-3) if len(cs) else (np.zeros(0), None, None)
        assert np.all(np.isfinite(e))
    dyn = np.array([b.type == 2 for b in cube_scene.bodies])
    # gravity pulls the dynamic cubes down on average
    assert (sim.pose.reshape(-1, 6)[dyn, 1] - y0[dyn]).mean() < 0
