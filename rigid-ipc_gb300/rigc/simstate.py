"""Simulation runs with the reference's state output, checkpoints and resume.

SimState follows src/SimState.cpp: a scene in the reference's JSON format is
stepped with the device time step (rigc_sim_step), each step's state is
appended to a state sequence (RigidBodyProblem::state,
src/physics/rigid_body_problem.cpp:107-150), the step's statistics are kept
(SimState::save_simulation_step, src/SimState.cpp:404-418: step timings,
Newton iterations, contacts, minimum distance), and the whole run is saved as
the reference's results file (SimState::save_simulation,
src/SimState.cpp:422-457):

    {"args": <the scene>, "animation": {"state_sequence": [...]},
     "stats": {...}}

A checkpoint is the same file written every checkpoint_every steps
(src/SimState.cpp:345-352); load() resumes from a results or checkpoint file
as SimState::load_simulation does (src/SimState.cpp:97-120): the scene from
"args", then the last state of the sequence.  After every step the run
checks for intersections (RigidBodyProblem::detect_intersections through
rigc_detect_intersections) and records the steps that had any, which the
reference logs as errors.

State of a body: position and rotation (the pose: centre of mass and
rotation vector of the body's principal frame), linear velocity, angular
velocity (the body-frame omega with Qdot = Q [omega]x), Qdot (3 x 3) and
Qddot (zero: the implicit-Euler step does not use it).
"""
from __future__ import annotations

import json
import time

import numpy as np

from . import scene as S


def _vee(W):
    return np.array([W[2, 1] - W[1, 2], W[0, 2] - W[2, 0], W[1, 0] - W[0, 1]]) * 0.5


class SimState:
    """One simulation of a reference-format scene on the device.

    solver: keyword arguments of Context.sim_init (Newton tolerances and the
    like); the time step, gravity, dhat, dmin, friction and the CCD
    trajectory (distance_barrier_constraint.trajectory_type) come from the
    scene."""

    def __init__(self, spec, **solver):
        from . import Context

        self.args = json.loads(spec) if isinstance(spec, str) else json.loads(json.dumps(spec))
        self.scene = S.scene_from_json(self.args)
        self.ctx = Context(self.scene)
        self.solver = dict(solver)
        sc = self.scene
        V = sc.world_vertices(sc.poses())
        # the stiffness bounds take the bounding box of the scene as read,
        # also when a run is resumed from a later state
        self.bbox_diagonal = float(np.linalg.norm(V.max(0) - V.min(0)))
        self._init(sc.poses().reshape(-1, 6), sc.velocities().reshape(-1, 6),
                   np.concatenate([b.Qdot.reshape(-1) for b in sc.bodies]).reshape(-1, 9))
        self.state_sequence = [self.state()]
        self.step_timings, self.solver_iterations = [], []
        self.num_contacts, self.step_minimum_distances = [], []
        self.intersecting_steps = []

    def _init(self, poses, velocities, Qdot):
        sc = self.scene
        solver = dict(self.solver)
        solver.setdefault("trajectory", sc.trajectory)
        self.ctx.sim_init(sc.timestep, sc.gravity, sc.dhat, sc.dmin,
                          coefficient_friction=sc.friction, poses=poses, velocities=velocities,
                          Qdot=Qdot, world_bbox_diagonal=self.bbox_diagonal, **solver)

    @property
    def num_steps(self):
        return len(self.state_sequence) - 1

    def state(self):
        """RigidBodyProblem::state: per-body pose and velocities, momenta and
        energies of the current state."""
        sc = self.scene
        P, V, Q, _ = self.ctx.sim_state()
        g = np.asarray(sc.gravity, dtype=np.float64)
        rbs = []
        p_lin = np.zeros(3)
        L_ang = np.zeros(3)
        T = 0.0
        G = 0.0
        for b, body in enumerate(sc.bodies):
            R = S.rotvec_to_matrix(P[b, 3:6])
            Qd = Q[b].reshape(3, 3)
            w = _vee(R.T @ Qd)
            rbs.append({"position": P[b, :3].tolist(), "rotation": P[b, 3:6].tolist(),
                        "linear_velocity": V[b, :3].tolist(), "angular_velocity": w.tolist(),
                        "Qdot": Qd.tolist(), "Qddot": np.zeros((3, 3)).tolist()})
            m = float(body.mass)
            I = np.asarray(body.moment_of_inertia, dtype=np.float64)
            p_lin += m * V[b, :3]
            L_ang += I * w
            T += 0.5 * m * float(V[b, :3] @ V[b, :3]) + 0.5 * float(w @ (I * w))
            fixed = np.asarray(body.is_dof_fixed, dtype=bool).reshape(-1)
            if not (fixed[0] and fixed[1]):
                G -= m * float(g @ P[b, :3])
        return {"rigid_bodies": rbs, "linear_momentum": p_lin.tolist(),
                "angular_momentum": L_ang.tolist(), "kinetic_energy": T, "potential_energy": G}

    def simulation_step(self):
        """One time step, its state and statistics; True when the new poses
        are intersection-free."""
        t = time.perf_counter()
        st = self.ctx.sim_step(1)
        self.step_timings.append(time.perf_counter() - t)
        self.solver_iterations.append(int(st["newton_iterations"]))
        P, _, _, _ = self.ctx.sim_state()
        x = P.reshape(-1)
        cs = self.ctx.construct_constraint_set(x, self.scene.dhat, self.scene.dmin)
        self.num_contacts.append(len(cs["type"]))
        self.step_minimum_distances.append(
            self.ctx.compute_min_distance(x, self.scene.dhat, self.scene.dmin))
        self.state_sequence.append(self.state())
        ok = self.ctx.detect_intersections(x) == 0
        if not ok:
            self.intersecting_steps.append(self.num_steps)
        return ok

    def run(self, steps=None, out=None, checkpoint_every=None):
        """Step to the scene's end (or `steps` more steps), writing a
        checkpoint '<out without .json>-chkpt<step>.json' every
        checkpoint_every steps and the results to `out` at the end."""
        steps = self.scene.num_steps - self.num_steps if steps is None else steps
        base = out[:-5] if out and out.endswith(".json") else out
        for i in range(steps):
            self.simulation_step()
            if (out and checkpoint_every and (i + 1) % checkpoint_every == 0
                    and i + 1 < steps):
                self.save(f"{base}-chkpt{self.num_steps:05d}.json")
        if out:
            self.save(out)
        return self

    def results(self):
        sc = self.scene
        stats = {"dim": 3, "num_bodies": sc.num_bodies, "num_vertices": sc.num_vertices,
                 "num_edges": int(len(sc.edges)), "num_faces": int(len(sc.faces)),
                 "num_timesteps": sc.num_steps, "step_timings": self.step_timings,
                 "solver_iterations": self.solver_iterations, "num_contacts": self.num_contacts,
                 "step_minimum_distances": self.step_minimum_distances,
                 "intersecting_steps": self.intersecting_steps}
        return {"args": self.args, "animation": {"state_sequence": self.state_sequence},
                "stats": stats}

    def save(self, path):
        with open(path, "w") as f:
            json.dump(self.results(), f)

    @classmethod
    def load(cls, results, **solver):
        """Resume from a results or checkpoint file (a path, text or dict):
        the scene from "args", the state from the last entry of the state
        sequence, the statistics from "stats"."""
        if isinstance(results, str) and not results.lstrip().startswith("{"):
            with open(results) as f:
                results = json.load(f)
        elif isinstance(results, str):
            results = json.loads(results)
        sim = cls(results["args"], **solver)
        seq = results["animation"]["state_sequence"]
        sim.state_sequence = list(seq)
        stats = results.get("stats", {})
        sim.step_timings = list(stats.get("step_timings", []))
        sim.solver_iterations = list(stats.get("solver_iterations", []))
        sim.num_contacts = list(stats.get("num_contacts", []))
        sim.step_minimum_distances = list(stats.get("step_minimum_distances", []))
        sim.intersecting_steps = list(stats.get("intersecting_steps", []))
        last = seq[-1]["rigid_bodies"]
        P = np.array([rb["position"] + rb["rotation"] for rb in last], dtype=np.float64)
        V = np.array([rb["linear_velocity"] + rb["angular_velocity"] for rb in last],
                     dtype=np.float64)
        Q = np.array([np.asarray(rb["Qdot"], dtype=np.float64).reshape(-1) for rb in last])
        sim._init(P, V, Q)
        return sim
