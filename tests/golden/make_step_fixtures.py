"""Oracle trajectories of the device time step's parity tests, as a fixture.

Runs of the oracle's restated IPC time step (implicit Euler, Newton with the
CCD-bounded line search, as DistanceBarrierRBProblem::simulation_step runs
it):

* cubes: the 27-cube lattice of the small plain configuration (seeded
  rotations and velocities, static plane, dt 0.01, dhat 1e-3, friction off),
  all 100 steps -- the cubes land on the plane around step 30 -- with the
  number of crossing (edge, face) pairs (RigidBodyProblem::
  detect_intersections) and the minimum distance after every step;
* cubes_tight: the same 100 steps with every Newton solve converged to
  rounding (velocity tolerance 1e-10 absolute, up to 8 full Newton steps
  after the line search stalls, CCD step bound 0.8 toi: the settings of the
  differentiation form).  With the reference's default tolerance (1e-2) a
  perturbation of 1e-15 in the initial poses grows to 1e-8 by step 11 and
  to 1e-2 by step 39 (the iterates are not converged, so rounding changes
  the Newton decisions).  With these settings it stays below 1e-13 until
  the landing steps, jumps to ~2e-8 in one of them and then grows linearly
  (a difference of ~1e-7 m/s in a frictionless sliding velocity) to ~1e-6
  by step 100;
* cubes_tight_branches: that sensitivity, resolved: the landing step where
  the jump happens ends its Newton solve at one of two iterations (the line
  search compares energies at the rounding level), and the two outcomes
  differ by 2e-8; the runs from initial poses perturbed by 1e-15 N(0, 1)
  (four seeds) that took the other outcome, with their minimum distances.
  A run that differs from the oracle's only in rounding follows one of
  these trajectories (to ~1e-13 per step), not necessarily the unperturbed
  one;
* cubes_pl_tight: the cubes_tight run with the line search's CCD on the
  piecewise-linear trajectory (the reference's JSON default), 40 steps
  through the landings; a 1e-15 perturbation of the start poses stays below
  2e-13 over them;
* pair: two cubes landing on the plane and sliding into each other with
  friction (mu 0.5), 10 steps;
* pile: 8 subdivision-3 icospheres in a seeded contact pile (2e-4 m gaps)
  with their seeded velocities and friction (mu 0.5), 2 steps.

Each run stores a digest of its inputs (rest vertices, initial poses and
velocities), so a test can tell whether its machine built the same scene.
Run from the repository root: python tests/golden/make_step_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "rigid-ipc_gb300"), os.path.join(ROOT, "oracle"), ROOT,
          os.path.join(ROOT, "tests"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

from make_headline_fixture import digest  # noqa: E402

OUT = os.path.join(HERE, "step_trajectories.npz")
H = 0.01
G = (0.0, -9.81, 0.0)
DHAT = 1e-3
CUBE_STEPS = 100
PAIR_STEPS = 10
PILE_STEPS = 2
MU = 0.5
TIGHT = dict(velocity_conv_tol=1e-10, velocity_conv_tol_abs=1, newton_polish=8, ccd_rescale=0.8)


def cubes_scene():
    from rigc import scene as S

    return S.scene_from_json(S.spec_cubes(0))


def pair_scene():
    from rigc import scene as S

    from test_adjoint_oracle import contact_pair_spec

    return S.scene_from_json(contact_pair_spec(3))


def pile_scene():
    """8 icospheres in a seeded contact pile: the scene and its start poses."""
    from rigc import scene as S

    sc = S.scene_from_json(S.spec_icospheres(seed=1, n=8, box=(2.5, 4.0, 2.5)))
    return sc, S.packed_pile_poses(sc, seed=1)


def inputs_digest(sc, x0):
    return digest(sc.rest_vertices, np.asarray(x0, np.float64), sc.velocities())


PL_STEPS = 40


def run(sc, steps, x0=None, mu=0.0, probes=False, **solver):
    import oracle as O

    O.build()
    sim = O.OracleSim(sc, h=H, gravity=G, dhat=DHAT, mu=mu, **solver)
    if x0 is not None:
        # start from x0; the world bounding-box diagonal (the barrier
        # stiffness bounds) is the start poses', as the device time step
        # takes it
        sim.pose[:] = x0
        V = sc.world_vertices(sim.pose)
        sim.bbox_diagonal = float(np.linalg.norm(V.max(0) - V.min(0)))
    o = O.OracleScene(sc)
    poses, kappa, crossings, md = [sim.pose.copy()], [], [], []
    for _ in range(steps):
        sim.step()
        poses.append(sim.pose.copy())
        kappa.append(sim.kappa.value)
        if probes:
            crossings.append(o.detect_intersections(sim.pose))
            md.append(o.min_distance(sim.pose, DHAT))
    return (np.array(poses), np.array(kappa), np.array(crossings, np.int64),
            np.array(md, np.float64))


def main():
    out = {}
    sc = cubes_scene()
    out["cubes_digest"] = inputs_digest(sc, sc.poses())
    (out["cubes_poses"], out["cubes_kappa"], out["cubes_crossings"],
     out["cubes_min_distance"]) = run(sc, CUBE_STEPS, probes=True)
    sc = pair_scene()
    out["pair_digest"] = inputs_digest(sc, sc.poses())
    out["pair_poses"], out["pair_kappa"], _, _ = run(sc, PAIR_STEPS, mu=MU)
    sc, x0 = pile_scene()
    out["pile_digest"] = inputs_digest(sc, x0)
    out["pile_poses"], out["pile_kappa"], _, _ = run(sc, PILE_STEPS, x0=x0, mu=MU)
    sc = cubes_scene()
    out["cubes_tight_digest"] = out["cubes_digest"]
    (out["cubes_tight_poses"], out["cubes_tight_kappa"], out["cubes_tight_crossings"],
     out["cubes_tight_min_distance"]) = run(sc, CUBE_STEPS, probes=True, **TIGHT)
    add_branches(out)
    add_pl(out)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: crossings per cube step {out['cubes_crossings'].max()}, "
          f"{out['cubes_tight_crossings'].max()} (tight)")


def add_pl(out):
    """cubes_pl_tight_poses / _crossings / _min_distance: the converged run
    with the piecewise-linear line-search CCD."""
    sc = cubes_scene()
    (out["cubes_pl_tight_poses"], _, out["cubes_pl_tight_crossings"],
     out["cubes_pl_tight_min_distance"]) = run(sc, PL_STEPS, probes=True, trajectory=1, **TIGHT)


BRANCH_SEEDS = (1, 2, 3, 4)


def _perturbed_run(seed):
    sc = cubes_scene()
    x0 = sc.poses() + 1e-15 * np.random.default_rng(seed).standard_normal(sc.poses().shape)
    poses, _, _, md = run(sc, CUBE_STEPS, x0=x0, probes=True, **TIGHT)
    return poses, md


def add_branches(out):
    """cubes_tight_branches / cubes_tight_branches_min_distance: the
    perturbed runs (one process per seed) that leave the unperturbed one by
    more than 1e-10 at some step, one per distinct trajectory."""
    import multiprocessing as mp

    with mp.get_context("spawn").Pool(len(BRANCH_SEEDS)) as pool:
        runs = pool.map(_perturbed_run, BRANCH_SEEDS)
    kept = [out["cubes_tight_poses"]]
    poses, md = [], []
    for p, m in runs:
        if min(np.abs(p[1:] - k[1:]).max() for k in kept) > 1e-10:
            kept.append(p)
            poses.append(p)
            md.append(m)
        print("seed run: largest difference to the unperturbed run",
              np.abs(p - out["cubes_tight_poses"]).max())
    out["cubes_tight_branches"] = np.array(poses).reshape(-1, *out["cubes_tight_poses"].shape)
    out["cubes_tight_branches_min_distance"] = np.array(md).reshape(-1, CUBE_STEPS)


if __name__ == "__main__":
    if "--pl" in sys.argv:
        # only the piecewise-linear entries, added to the existing file
        out = dict(np.load(OUT))
        add_pl(out)
        np.savez_compressed(OUT, **out)
        print("piecewise-linear run", out["cubes_pl_tight_poses"].shape)
    elif "--branches" in sys.argv:
        # only the branch entries, added to the existing file
        out = dict(np.load(OUT))
        add_branches(out)
        np.savez_compressed(OUT, **out)
        print(f"{len(out['cubes_tight_branches'])} branch trajectories")
    else:
        main()
