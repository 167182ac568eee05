"""Central finite differences of the oracle's simulator for the
differentiation workload, kept as a fixture for the GPU adjoint test.

Run from the repository root (CPU only; about ten minutes on 8 cores):

    python tests/golden/make_adjoint_fixture.py

and, for the central differences of every parameter (1,536 rollouts, about
an hour and a half on 8 cores):

    python tests/golden/make_adjoint_fixture.py --all-parameters

Workload: 64 unit cubes in a 4 x 4 x 4 lattice (spacing 1.05 m, seeded
rotations, lowest layer 0.5 m above a static 20 x 20 m plane, at rest),
50 implicit-Euler steps of 0.01 s, dhat = 1e-3, no friction; the lowest
layer lands on the plane around step 30 and the upper layers on it after.
Loss: |c_0(T) - (3, 0, 0.5)|^2 for cube 0's centre.  Parameters: the 64
cubes' initial linear and angular velocities (omega in body coordinates,
Qdot0 = R(theta0) [omega]x), 384 values.

Solver settings of the differentiable rollout: velocity convergence 1e-10
m/s (absolute), 8 Newton polish steps, CCD step bound 0.8 toi.

Output tests/golden/adjoint_cube_lattice.npz: the scene's bodies as arrays
(scene_from_arrays rebuilds them bit for bit), the loss, the oracle adjoint
gradient (64 x 6 over (v, omega); the plane's row is zero), seeded random
directions, the central differences of the loss along them at h = 1e-6 and
2e-6, their Richardson extrapolation (4 D(h) - D(2h)) / 3, and the oracle's
iteration counts.

The landings make the loss stiff: central differences at h = 1e-6 carry a
truncation error of about 2e-5 relative here, shrinking as h^2 (at h = 1e-7
they agree with the adjoint to 2e-7), so the extrapolated differences, with
an O(h^4) error, are the ones to compare with at 1e-5.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

H = 0.01
G = (0.0, -9.81, 0.0)
DHAT = 1e-3
STEPS = 50
TARGET = np.array([3.0, 0.0, 0.5])
DIFF = dict(velocity_conv_tol=1e-10, velocity_conv_tol_abs=1, newton_polish=8, ccd_rescale=0.8)
FD_H = 1e-6
NUM_DIRECTIONS = 4
SEED = 0


def _paths():
    for p in (os.path.join(ROOT, "rigid-ipc_gb300"), os.path.join(ROOT, "oracle"),
              os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)


def lattice_scene():
    _paths()
    from rigc import scene as S

    return S.scene_from_json(S.spec_cube_lattice(SEED))


SCENE_KEYS = ("vertices", "edges", "faces", "faces_to_edges", "pose", "velocity", "mass",
              "moment_of_inertia", "is_dof_fixed", "type", "group_id", "r_max",
              "average_edge_length", "Qdot")


def scene_arrays(sc):
    """The scene's bodies as flat arrays (per-body arrays concatenated, with
    start offsets), so that a test rebuilds the very same bits on any machine."""
    out = {}
    for k in ("vertices", "edges", "faces", "faces_to_edges"):
        parts = [np.asarray(getattr(b, k)) for b in sc.bodies]
        out["body_" + k] = np.concatenate(parts)
        out["body_" + k + "_start"] = np.cumsum([0] + [len(p) for p in parts]).astype(np.int64)
    for k in SCENE_KEYS[4:]:
        out["body_" + k] = np.array([np.asarray(getattr(b, k)) for b in sc.bodies])
    return out


def scene_from_arrays(d):
    _paths()
    from rigc import scene as S

    nb = len(d["body_mass"])
    bodies = []
    for i in range(nb):
        kw = {}
        for k in SCENE_KEYS[:4]:
            a, b = d["body_" + k + "_start"][i], d["body_" + k + "_start"][i + 1]
            kw[k] = np.array(d["body_" + k][a:b])
        for k in SCENE_KEYS[4:]:
            v = d["body_" + k][i]
            kw[k] = np.array(v) if np.ndim(v) else v.item()
        bodies.append(S.RigidBody(name=f"body{i}", **kw))
    return S.Scene(bodies=bodies)


def directions(nb):
    rng = np.random.default_rng(1234)
    out = []
    for _ in range(NUM_DIRECTIONS):
        d = rng.normal(size=(nb, 6))
        d[nb - 1] = 0  # the static plane
        out.append(d)
    return np.array(out)


def _loss(dvel):
    _paths()
    import oracle as O
    from test_adjoint_oracle import qdot_of

    sc = lattice_scene()  # the same bits in every worker of this machine
    sim = O.OracleSim(sc, h=H, gravity=G, dhat=DHAT, **DIFF)
    nb = len(sim.mass)
    poses = sim.pose.reshape(nb, 6)
    vel = sim.vel.reshape(nb, 6) + dvel
    sim.vel = np.ascontiguousarray(vel.reshape(-1))
    sim.Qdot = np.ascontiguousarray(qdot_of(poses, vel[:, 3:]))
    sim.rollout(STEPS, record=False)
    c = sim.pose.reshape(nb, 6)[0, :3]
    return float(((c - TARGET) ** 2).sum())


def main():
    _paths()
    import oracle as O
    from test_adjoint_oracle import omega_gradient, qdot_of

    O.build()
    sc = lattice_scene()
    nb = sc.num_bodies
    t = time.time()
    sim = O.OracleSim(sc, h=H, gravity=G, dhat=DHAT, **DIFF)
    poses = sim.pose.reshape(nb, 6).copy()
    vel = sim.vel.reshape(nb, 6).copy()
    sim.Qdot = np.ascontiguousarray(qdot_of(poses, vel[:, 3:]))
    sim.rollout(STEPS, record=True)
    c = sim.pose.reshape(nb, 6)[0, :3]
    loss = float(((c - TARGET) ** 2).sum())
    dp = np.zeros((nb, 6))
    dp[0, :3] = 2 * (c - TARGET)
    gp, gv, gq = sim.backward(dp)
    grad = np.concatenate([gv[:, :3], omega_gradient(poses, gq)], 1)
    print(f"rollout + adjoint {time.time() - t:.1f}s, stats {sim.stats}, loss {loss:.12f}")
    D = directions(nb)
    hs = (FD_H, 2 * FD_H)
    jobs = [d * s * h for h in hs for d in D for s in (1.0, -1.0)]
    # one worker per perturbed rollout (the oracle's CCD threads inside each)
    with mp.get_context("spawn").Pool(min(len(jobs), max(1, (os.cpu_count() or 2) // 2))) as pool:
        losses = np.array(pool.map(_loss, jobs)).reshape(len(hs), len(D), 2)
    fd = np.array([(losses[i, :, 0] - losses[i, :, 1]) / (2 * h) for i, h in enumerate(hs)])
    fd_extrapolated = (4 * fd[0] - fd[1]) / 3
    ad = np.einsum("kbj,bj->k", D, grad)
    for k in range(len(D)):
        print(f"direction {k}: fd(h) {fd[0, k]:.12e} fd(2h) {fd[1, k]:.12e} "
              f"extrapolated {fd_extrapolated[k]:.12e} adjoint {ad[k]:.12e} "
              f"rel {abs(fd_extrapolated[k] - ad[k]) / abs(fd_extrapolated[k]):.2e}")
    np.savez_compressed(os.path.join(HERE, "adjoint_cube_lattice.npz"), loss=np.float64(loss),
                        grad=grad, directions=D, fd=fd[0], fd_2h=fd[1],
                        fd_extrapolated=fd_extrapolated, fd_h=np.float64(FD_H),
                        steps=np.int64(STEPS), seed=np.int64(SEED),
                        final_poses=sim.pose.reshape(nb, 6), stats=sim.stats,
                        **scene_arrays(sc))


FD_ALL_OUT = os.path.join(HERE, "adjoint_cube_lattice_fd.npz")


def _loss_param(job):
    """Loss with one initial velocity component (body b, component k)
    shifted by delta."""
    b, k, delta = job
    d = np.zeros((65, 6))
    d[b, k] = delta
    return _loss(d)


def main_all_parameters(workers):
    """Central differences of the loss for every one of the 384 parameters
    (the 64 cubes' initial linear and angular velocities) at h = 1e-6 and at
    h / 2, each from two rollouts of the oracle: 1,536 rollouts, spread over
    `workers` processes.  Written to adjoint_cube_lattice_fd.npz: fd_h and
    fd_h2 (64 x 6, the cubes' rows in the order of the scene), their
    Richardson extrapolation (4 D(h/2) - D(h)) / 3, the step sizes."""
    _paths()
    import oracle as O

    O.build()
    sc = lattice_scene()
    nb = sc.num_bodies
    hs = (FD_H, FD_H / 2)
    jobs = [(b, k, s * h) for h in hs for b in range(nb - 1) for k in range(6)
            for s in (1.0, -1.0)]
    t = time.time()
    with mp.get_context("spawn").Pool(workers) as pool:
        losses = np.array(pool.map(_loss_param, jobs, chunksize=4))
    losses = losses.reshape(len(hs), nb - 1, 6, 2)
    fd = np.array([(losses[i, :, :, 0] - losses[i, :, :, 1]) / (2 * h) for i, h in enumerate(hs)])
    np.savez_compressed(FD_ALL_OUT, fd_h=fd[0], fd_h2=fd[1],
                        fd_extrapolated=(4 * fd[1] - fd[0]) / 3, h=np.float64(hs[0]),
                        steps=np.int64(STEPS), seed=np.int64(SEED))
    print(f"wrote {FD_ALL_OUT}: {len(jobs)} rollouts in {time.time() - t:.0f}s")


if __name__ == "__main__":
    if "--all-parameters" in sys.argv:
        main_all_parameters(int(os.environ.get("FD_WORKERS", max(1, (os.cpu_count() or 2) - 1))))
    else:
        main()
