"""The device adjoint (rigc_sim_rollout / rigc_sim_backward through the C ABI,
and the torch.autograd.Function over it) against the oracle's adjoint and
against central finite differences (h = 1e-6) of the oracle's simulator.

Bars: poses after the rollout within 1e-8 of the oracle's; gradients within
1e-6 (max-norm relative) of the oracle's adjoint, within 1e-5 relative of
the finite differences along random directions, within 1e-7 of the largest
component of the extrapolated differences in every one of the differentiation
workload's 384 parameters; checkpoint intervals give
bit-identical gradients (the recomputed segments are bit-identical)."""
import numpy as np
import pytest

from test_adjoint_oracle import (DHAT, DIFF, FD_RTOL, G, H, STEPS, TARGET, contact_pair,
                                 fd_directional, fd_directions, omega_gradient,
                                 oracle_gradient, oracle_rollout, qdot_of)

pytestmark = pytest.mark.gpu


def gpu_gradient(sc, steps=STEPS, every=10):
    """(final poses, dL/d(v, omega) nb x 6, context) through the C ABI."""
    import rigc

    ctx = rigc.Context(sc)
    nb = sc.num_bodies
    poses = sc.poses().reshape(nb, 6)
    vel = sc.velocities().reshape(nb, 6)
    ctx.sim_init(H, G, DHAT, poses=poses, velocities=vel, Qdot=qdot_of(poses, vel[:, 3:]), **DIFF)
    ctx.sim_rollout(steps, every)
    P, V, Q, _ = ctx.sim_state()
    dp = np.zeros((nb, 6))
    dp[0, :3] = 2 * (P[0, :3] - TARGET)
    gp, gv, gq = ctx.sim_backward(dp)
    return P, np.concatenate([gv[:, :3], omega_gradient(poses, gq)], 1), ctx


@pytest.fixture(scope="module")
def pair():
    return contact_pair()


@pytest.fixture(scope="module")
def oracle_pair(oracle, pair):
    return oracle_gradient(oracle, pair)


@pytest.fixture(scope="module")
def gpu_pair(pair):
    return gpu_gradient(pair)


def test_rollout_matches_oracle(pair, oracle_pair, gpu_pair):
    L, g_o, sim = oracle_pair
    P, g, ctx = gpu_pair
    nb = pair.num_bodies
    assert np.abs(P - sim.pose.reshape(nb, 6)).max() <= 1e-8


def test_gradient_matches_oracle_adjoint(oracle_pair, gpu_pair):
    _, g_o, _ = oracle_pair
    _, g, _ = gpu_pair
    assert np.abs(g - g_o).max() <= 1e-6 * np.abs(g_o).max()


def test_gradient_matches_finite_differences(oracle, pair, gpu_pair):
    _, g, _ = gpu_pair
    dyn = np.array([b.type == 2 for b in pair.bodies])
    for d in fd_directions(pair.num_bodies, dyn):
        ad = float((g * d).sum())
        fd = fd_directional(oracle, pair, d)
        assert abs(ad - fd) <= FD_RTOL * abs(fd), (ad, fd)


def test_checkpoint_interval_bit_identical(pair, gpu_pair):
    _, g10, _ = gpu_pair
    for every in (1, 3):
        _, g, _ = gpu_gradient(pair, every=every)
        assert np.array_equal(g, g10)


def test_backward_leaves_final_state(pair):
    P, _, ctx = gpu_gradient(pair)
    P2, V2, Q2, _ = ctx.sim_state()
    assert np.array_equal(P, P2)
    # and a second backward gives the same gradient
    nb = pair.num_bodies
    dp = np.zeros((nb, 6))
    dp[0, :3] = 2 * (P[0, :3] - TARGET)
    a = ctx.sim_backward(dp)
    b = ctx.sim_backward(dp)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_free_fall_closed_form():
    from rigc import meshes, scene as S

    V, F = meshes.cube()
    sc = S.Scene(bodies=[S.make_body(V, F, position=(0, 5, 0), linear_velocity=(0.3, 1.0, -0.2))])
    T = 5
    P, g, _ = gpu_gradient(sc, steps=T, every=2)
    assert np.allclose(g[0, :3], 2 * (P[0, :3] - TARGET) * T * H, rtol=1e-12, atol=1e-14)
    assert np.abs(g[0, 3:]).max() <= 1e-12


def test_autograd_function(pair, gpu_pair):
    """loss.backward() through rigc.adjoint.DifferentiableSimulation gives the
    C-ABI gradient; omega's gradient flows through qdot_from_omega in torch."""
    import torch

    from rigc.adjoint import DifferentiableSimulation, qdot_from_omega

    _, g_ref, _ = gpu_pair
    sim = DifferentiableSimulation(pair, H, G, DHAT, checkpoint_every=10, **DIFF)
    nb = pair.num_bodies
    dev = "cuda"
    poses = torch.as_tensor(pair.poses().reshape(nb, 6), dtype=torch.float64, device=dev)
    vel0 = pair.velocities().reshape(nb, 6)
    v = torch.as_tensor(vel0[:, :3], dtype=torch.float64, device=dev).requires_grad_()
    w = torch.as_tensor(vel0[:, 3:], dtype=torch.float64, device=dev).requires_grad_()
    P, V, Q = sim(poses, torch.cat([v, w], 1), qdot_from_omega(poses, w), STEPS)
    loss = ((P[0, :3] - torch.as_tensor(TARGET, dtype=torch.float64, device=dev)) ** 2).sum()
    loss.backward()
    g = torch.cat([v.grad, w.grad], 1).cpu().numpy()
    assert np.abs(g - g_ref).max() <= 1e-10 * np.abs(g_ref).max()
    assert sim.stats["newton_iterations"] > 0


def test_backward_rejects_friction(pair):
    import rigc

    ctx = rigc.Context(pair)
    ctx.sim_init(H, G, DHAT, coefficient_friction=0.5, **DIFF)
    ctx.sim_rollout(1, 1)
    with pytest.raises(RuntimeError):
        ctx.sim_backward(np.zeros((pair.num_bodies, 6)))


def test_cube_lattice_adjoint_matches_fixture():
    """The differentiation workload (64 cubes landing on a plane, 50 steps,
    384 velocity parameters): the device gradient against the oracle's
    adjoint and against central differences (h = 1e-6) of the oracle's
    simulator along random directions (tests/golden/adjoint_cube_lattice.npz)
    and in every one of the 384 parameters at h = 1e-6 and h / 2
    (tests/golden/adjoint_cube_lattice_fd.npz)."""
    import os

    import make_adjoint_fixture as F

    fx = np.load(os.path.join(os.path.dirname(F.__file__), "adjoint_cube_lattice.npz"))
    sc = F.scene_from_arrays(fx)
    import rigc

    ctx = rigc.Context(sc)
    nb = sc.num_bodies
    poses = sc.poses().reshape(nb, 6)
    vel = sc.velocities().reshape(nb, 6)
    ctx.sim_init(F.H, F.G, F.DHAT, poses=poses, velocities=vel, Qdot=qdot_of(poses, vel[:, 3:]),
                 **F.DIFF)
    ctx.sim_rollout(int(fx["steps"]), 10)
    P, _, _, _ = ctx.sim_state()
    loss = float(((P[0, :3] - F.TARGET) ** 2).sum())
    assert np.abs(P - fx["final_poses"]).max() <= 1e-8
    assert abs(loss - float(fx["loss"])) <= 1e-10 * float(fx["loss"])
    dp = np.zeros((nb, 6))
    dp[0, :3] = 2 * (P[0, :3] - F.TARGET)
    gp, gv, gq = ctx.sim_backward(dp)
    g = np.concatenate([gv[:, :3], omega_gradient(poses, gq)], 1)
    assert np.abs(g - fx["grad"]).max() <= 1e-6 * np.abs(fx["grad"]).max()
    for d, fd, fd_x in zip(fx["directions"], fx["fd"], fx["fd_extrapolated"]):
        ad = float((g * d).sum())
        # extrapolated central differences (h = 1e-6, 2e-6) at the 1e-5 bar;
        # the plain ones at h = 1e-6 are truncation-limited (~2e-5) here
        assert abs(ad - fd_x) <= FD_RTOL * abs(fd_x), (ad, fd_x)
        assert abs(ad - fd) <= 1e-4 * abs(fd), (ad, fd)
    # every one of the 384 parameters: central differences of the oracle's
    # simulator at h = 1e-6 and h / 2 (adjoint_cube_lattice_fd.npz) and
    # their extrapolation
    fd_all = np.load(os.path.join(os.path.dirname(F.__file__), "adjoint_cube_lattice_fd.npz"))
    ga = g[:64]
    scale = np.abs(fd_all["fd_extrapolated"]).max()
    assert np.abs(ga - fd_all["fd_h"]).max() <= 1e-5 * scale
    assert np.abs(ga - fd_all["fd_h2"]).max() <= 3e-6 * scale
    assert np.abs(ga - fd_all["fd_extrapolated"]).max() <= 1e-7 * scale
