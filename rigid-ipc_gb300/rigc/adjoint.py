"""Differentiable rollouts: the device time step and its adjoint exposed as a
``torch.autograd.Function``.

The forward pass runs ``num_steps`` implicit-Euler IPC steps on the GPU
(``rigc_sim_rollout``, checkpoints every ``checkpoint_every`` steps); the
backward pass differentiates every converged step implicitly on the GPU
(``rigc_sim_backward``: H lambda = dL/dx* with the assembled unprojected
Hessian, segments recomputed from their checkpoints).  The reference has no
adjoint; its state and step are those of DistanceBarrierRBProblem::
simulation_step (src/problems/distance_barrier_rb_problem.cpp:118-143) and
RigidBodyProblem::take_step (src/physics/rigid_body_problem.cpp:225-262).

State per body: pose [p, theta] (6), velocities [v world, omega body] (6)
and Qdot = dR/dt (9, row-major); the step consumes p, theta, v and Qdot.
``qdot_from_omega`` builds Qdot = R(theta) [omega]x as the reference does
at start-up (src/physics/rigid_body.cpp:141), in torch, so gradients reach
omega (and theta) through it.
"""
from __future__ import annotations

import numpy as np
import torch

from . import Context

# settings under which each step converges and its gradient vanishes to
# rounding: tight velocity convergence, full Newton steps after the line
# search stalls, and a CCD step bound of 0.8 toi (so the first step into a
# contact does not end below the rigid CCD's resolution)
DIFF_DEFAULTS = dict(velocity_conv_tol=1e-10, velocity_conv_tol_abs=True, newton_polish=8,
                     ccd_rescale=0.8)


def hat(w: torch.Tensor) -> torch.Tensor:
    """[w]x for (..., 3) -> (..., 3, 3)."""
    z = torch.zeros_like(w[..., 0])
    return torch.stack([torch.stack([z, -w[..., 2], w[..., 1]], -1),
                        torch.stack([w[..., 2], z, -w[..., 0]], -1),
                        torch.stack([-w[..., 1], w[..., 0], z], -1)], -2)


def rotation_matrix(theta: torch.Tensor) -> torch.Tensor:
    """R = I + sinc|t| [t]x + (1 - cos|t|) / |t|^2 [t]x^2 (Pose::
    construct_rotation_matrix, src/physics/pose.tpp:203-218), differentiable
    at t = 0."""
    t2 = (theta * theta).sum(-1, keepdim=True)
    small = t2 < 1e-16
    t2s = torch.where(small, torch.ones_like(t2), t2)
    n = t2s.sqrt()
    a = torch.where(small, 1 - t2 / 6, torch.sin(n) / n)
    b = torch.where(small, 0.5 - t2 / 24, (1 - torch.cos(n)) / t2s)
    K = hat(theta)
    eye = torch.eye(3, dtype=theta.dtype, device=theta.device).expand_as(K)
    return eye + a[..., None] * K + b[..., None] * (K @ K)


def qdot_from_omega(poses: torch.Tensor, omega: torch.Tensor) -> torch.Tensor:
    """Qdot = R(theta) [omega]x with omega in body coordinates, nb x 9."""
    R = rotation_matrix(poses[:, 3:6])
    return (R @ hat(omega)).reshape(-1, 9)


class Rollout(torch.autograd.Function):
    """(poses, velocities, Qdot) -> the same after num_steps device steps."""

    @staticmethod
    def forward(fctx, poses, velocities, Qdot, sim, num_steps, checkpoint_every):
        host = [t.detach().to("cpu", torch.float64).contiguous().numpy()
                for t in (poses, velocities, Qdot)]
        sim.context.sim_init(**sim.params, poses=host[0], velocities=host[1], Qdot=host[2])
        sim.stats = sim.context.sim_rollout(num_steps, checkpoint_every)
        sim.generation += 1
        fctx.sim = sim
        fctx.generation = sim.generation
        fctx.device = poses.device
        P, V, Q, _ = sim.context.sim_state()
        dev = dict(dtype=torch.float64, device=poses.device)
        return torch.as_tensor(P, **dev), torch.as_tensor(V, **dev), torch.as_tensor(Q, **dev)

    @staticmethod
    def backward(fctx, gP, gV, gQ):
        sim = fctx.sim
        if sim.generation != fctx.generation:
            raise RuntimeError("Rollout.backward: the simulation ran another rollout since this "
                               "one; call backward before the next forward")

        def host(g):
            return None if g is None else g.detach().to("cpu", torch.float64).contiguous().numpy()

        nb = sim.context.scene.num_bodies
        dp = host(gP) if gP is not None else np.zeros((nb, 6))
        gp, gv, gq = sim.context.sim_backward(dp, host(gV), host(gQ))
        dev = dict(dtype=torch.float64, device=fctx.device)
        return (torch.as_tensor(gp, **dev), torch.as_tensor(gv, **dev),
                torch.as_tensor(gq, **dev), None, None, None)


class DifferentiableSimulation:
    """A scene on the GPU whose rollouts torch can differentiate.

    ``sim(poses, velocities, Qdot, num_steps)`` returns the state after
    num_steps steps as float64 tensors; ``loss.backward()`` runs the device
    adjoint.  One tape per simulation: differentiate a rollout before
    starting the next.  Friction is not differentiated."""

    def __init__(self, scene, timestep, gravity, dhat, checkpoint_every=10, **params):
        if params.get("coefficient_friction", 0.0) > 0:
            raise ValueError("DifferentiableSimulation: friction is not differentiated")
        self.context = Context(scene)
        self.checkpoint_every = int(checkpoint_every)
        self.params = dict(timestep=timestep, gravity=tuple(gravity), dhat=dhat)
        self.params.update(DIFF_DEFAULTS)
        self.params.update(params)
        self.generation = 0
        self.stats = None

    def __call__(self, poses, velocities, Qdot, num_steps):
        return Rollout.apply(poses, velocities, Qdot, self, int(num_steps), self.checkpoint_every)
