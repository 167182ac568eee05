"""The device time step (rigc_sim_*) against the oracle's restated step:
the closed-form free fall, and the 27-cube scene over several steps (poses
within 1e-7: the Newton systems are solved by different methods, an LDL^T on
the CPU and preconditioned conjugate gradients to a 1e-12 residual on the
GPU, so the iterates agree to the solve accuracy, not bit for bit)."""
import numpy as np
import pytest

from test_step_oracle import G, H, free_cube

pytestmark = pytest.mark.gpu


def test_free_fall_gpu():
    import rigc

    sc = free_cube()
    ctx = rigc.Context(sc)
    ctx.sim_init(H, G, 1e-3)
    p = sc.poses()[:3].copy()
    v = sc.velocities()[:3].copy()
    for _ in range(3):
        ctx.sim_step(1)
        P, V, Q, k = ctx.sim_state()
        v = v + H * np.array(G)
        p = p + H * v
        assert np.allclose(P[0, :3], p, rtol=0, atol=1e-12)
        assert np.allclose(V[0, :3], v, rtol=0, atol=1e-10)


def test_cube_lattice_matches_oracle(oracle, cube_scene):
    import rigc

    nsteps = 4
    sim = oracle.OracleSim(cube_scene, h=H, gravity=G, dhat=1e-3)
    ctx = rigc.Context(cube_scene)
    ctx.sim_init(H, G, 1e-3)
    for k in range(nsteps):
        st_o = sim.step()
        st_g = ctx.sim_step(1)
        P, V, Q, kappa = ctx.sim_state()
        err = np.abs(P.reshape(-1) - sim.pose).max()
        assert err <= 1e-7, (k, err, st_o, st_g)
        assert kappa == pytest.approx(sim.kappa.value, rel=1e-12)
        assert np.abs(V.reshape(-1)[:] - sim.vel).reshape(-1, 6)[:, :3].max() <= 1e-5


def test_large_lattice_cg_graph_matches_oracle(oracle):
    """216 cubes (1296 free dofs): the Newton systems go to the conjugate
    gradient solver, whose iteration loop runs as one CUDA graph launch (a
    device-side while loop); poses after 2 steps against the oracle's dense
    LDL^T solve."""
    import rigc
    from rigc import scene as S

    sc = S.scene_from_json(S.spec_cubes(3, n=6, vel_sigma=0.5))
    sim = oracle.OracleSim(sc, h=H, gravity=G, dhat=1e-3)
    ctx = rigc.Context(sc)
    ctx.sim_init(H, G, 1e-3)
    cg = 0
    for k in range(2):
        st_o = sim.step()
        st_g = ctx.sim_step(1)
        cg += st_g["cg_iterations"]
        P, V, Q, kappa = ctx.sim_state()
        err = np.abs(P.reshape(-1) - sim.pose).max()
        assert err <= 1e-7, (k, err, st_o, st_g)
        assert kappa == pytest.approx(sim.kappa.value, rel=1e-12)
    assert cg > 0  # the CG path ran


def test_kinematic_bodies_match_oracle(oracle):
    """A kinematic cube (the augmented Lagrangian toward x0 + h v) pushing a
    dynamic one across a plane: device poses after 3 steps against the
    oracle's."""
    import rigc

    from test_kinematic_oracle import paddle_scene

    sc = paddle_scene()
    sim = oracle.OracleSim(sc, h=0.01, gravity=(0.0, -9.81, 0.0), dhat=1e-3)
    ctx = rigc.Context(sc)
    ctx.sim_init(0.01, (0.0, -9.81, 0.0), 1e-3)
    for _ in range(3):
        sim.step()
        ctx.sim_step(1)
        P, V, Q, k = ctx.sim_state()
        assert np.abs(P.reshape(-1) - sim.pose).max() <= 1e-7
    with pytest.raises(RuntimeError):  # kinematic bodies are not differentiated
        ctx.sim_rollout(1, 1)
        ctx.sim_backward(np.zeros((sc.num_bodies, 6)))
