"""The device time step (rigc_sim_*) against the oracle's restated step:
the closed-form free fall, a few steps of the 27-cube scene, of a 216-cube
lattice (the conjugate-gradient path) and of kinematic bodies (poses within
1e-7: the iterates agree to the accuracy of the Newton solves, not bit for
bit), and whole runs against the oracle's trajectories in
tests/golden/step_trajectories.npz at 1e-8."""
import os

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


def test_kinematic_schedule_matches_oracle(oracle):
    """A kinematic cube driven through its JSON pose list into a dynamic one,
    then by its velocity, static once kinematic_max_time has run out
    (rigc_sim_set_kinematic, set by sim_init from the scene): device poses
    against the oracle's after each of 8 steps, with the reference's solver
    settings, within 1e-6 (the kinematic targets are met to the augmented
    Lagrangian's progress tolerance, 0.999 of the step, and its discrete
    penalty and multiplier updates follow the iterates, so a rounding-level
    difference in a contact step can move the solution at that level; the
    same settings keep the first four steps within 1e-7); the body does not
    move after it became static."""
    import rigc

    from test_kinematic_oracle import scheduled_scene

    sc = scheduled_scene()
    sim = oracle.OracleSim(sc, h=0.01, gravity=(0.0, -9.81, 0.0), dhat=1e-3)
    ctx = rigc.Context(sc)
    ctx.sim_init(0.01, (0.0, -9.81, 0.0), 1e-3)
    frozen = None
    for k in range(8):
        sim.step()
        ctx.sim_step(1)
        P, V, Q, _ = ctx.sim_state()
        assert np.abs(P.reshape(-1) - sim.pose).max() <= (1e-7 if k < 4 else 1e-6), k
        if k >= 5:
            assert sim.type[1] == 0 and np.all(V[1] == 0)
            if frozen is None:
                frozen = P[1].copy()
            assert np.array_equal(P[1], frozen)
    with pytest.raises(RuntimeError):  # only kinematic bodies have a schedule
        ctx.sim_set_kinematic(2, 1.0, [])


# ---------------------------------------------------------------------------
# whole runs against the oracle's trajectories (tests/golden/
# step_trajectories.npz, made by make_step_fixtures.py), at the 1e-8 pose
# bar, with the end-of-step intersection check

POSE_ATOL = 1e-8
FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                       "step_trajectories.npz")


def _fixture(key, sc, x0):
    import make_step_fixtures as SF

    fx = np.load(FIXTURE)
    if SF.inputs_digest(sc, x0) != str(fx[key + "_digest"]):
        pytest.skip("this machine builds a different scene (floating-point set-up differs)")
    return fx


def test_cube_lattice_whole_run_matches_oracle():
    """All 100 steps of the 27-cube lattice (landings from step ~20) with
    every Newton solve converged to rounding: after every step the poses are
    within 1e-8 of one of the oracle's trajectories -- the unperturbed run or
    a run from start poses perturbed by 1e-15 that took the other outcome of
    the landing step whose Newton solve ends at one of two iterations (the
    two outcomes differ by 2e-8); no crossing edge and face after any step on
    either side; the minimum distance of the matched oracle run."""
    import rigc

    import make_step_fixtures as SF

    sc = SF.cubes_scene()
    fx = _fixture("cubes_tight", sc, sc.poses())
    runs = [fx["cubes_tight_poses"], *fx["cubes_tight_branches"]]
    mds = [fx["cubes_tight_min_distance"], *fx["cubes_tight_branches_min_distance"]]
    assert len(runs) >= 2  # the fixture resolves the two outcomes
    ctx = rigc.Context(sc)
    ctx.sim_init(SF.H, SF.G, SF.DHAT, **SF.TIGHT)
    assert fx["cubes_tight_crossings"].max() == 0
    landed = 0
    for k in range(SF.CUBE_STEPS):
        ctx.sim_step(1)
        P, V, Q, kappa = ctx.sim_state()
        x = P.reshape(-1)
        errs = [np.abs(x - r[k + 1]).max() for r in runs]
        j = int(np.argmin(errs))
        assert errs[j] <= POSE_ATOL, (k, errs)
        assert ctx.detect_intersections(x) == 0, k
        md_o = mds[j][k]
        md = ctx.compute_min_distance(x, SF.DHAT)
        assert (md < 0) == (md_o < 0), k
        if md_o > 0:
            landed += 1
            assert abs(md - md_o) <= 1e-9, (k, md, md_o)
    assert landed > 20  # the cubes rest on the plane for the last steps


def test_cube_lattice_piecewise_linear_matches_oracle():
    """The converged 27-cube run with the line search's CCD on the
    piecewise-linear trajectory (the reference's JSON default): poses within
    1e-10 of the oracle's after each of 40 steps through the landings (a
    1e-15 perturbation of the oracle's start stays below 2e-13 here), no
    crossing edge and face after any step, the oracle's minimum distance."""
    import rigc

    import make_step_fixtures as SF

    sc = SF.cubes_scene()
    fx = _fixture("cubes", sc, sc.poses())
    ctx = rigc.Context(sc)
    ctx.sim_init(SF.H, SF.G, SF.DHAT, trajectory="piecewise_linear", **SF.TIGHT)
    assert fx["cubes_pl_tight_crossings"].max() == 0
    for k in range(SF.PL_STEPS):
        ctx.sim_step(1)
        P, V, Q, kappa = ctx.sim_state()
        x = P.reshape(-1)
        err = np.abs(x - fx["cubes_pl_tight_poses"][k + 1]).max()
        assert err <= 1e-10, (k, err)
        assert ctx.detect_intersections(x) == 0, k
        md_o = fx["cubes_pl_tight_min_distance"][k]
        md = ctx.compute_min_distance(x, SF.DHAT)
        assert (md < 0) == (md_o < 0), k
        if md_o > 0:
            assert abs(md - md_o) <= 1e-9, (k, md, md_o)


def test_piecewise_linear_rejected_on_batched_context():
    import rigc
    from rigc import scene as S

    scenes = [S.scene_from_json(S.spec_cubes(seed)) for seed in range(2)]
    big, sob = S.concat_scenes(scenes)
    ctx = rigc.Context(big, scene_of_body=sob)
    with pytest.raises(RuntimeError):
        ctx.sim_init(0.01, (0, -9.81, 0), 1e-3, trajectory="piecewise_linear")


def test_cube_lattice_default_solver():
    """The same run with the reference's default Newton tolerance
    (velocity_conv_tol 1e-2): the iterates are not converged, so any change
    of rounding (1e-15 in the start poses) grows tenfold per contact step --
    to 1e-8 by step 11 in the oracle itself.  The first 8 steps match the
    oracle's within 1e-8; over all 100 steps the run stays intersection-free
    and the cubes come to rest on the plane in the oracle's three layers."""
    import rigc

    import make_step_fixtures as SF

    sc = SF.cubes_scene()
    fx = _fixture("cubes", sc, sc.poses())
    ctx = rigc.Context(sc)
    ctx.sim_init(SF.H, SF.G, SF.DHAT)
    assert fx["cubes_crossings"].max() == 0
    for k in range(SF.CUBE_STEPS):
        ctx.sim_step(1)
        P, V, Q, kappa = ctx.sim_state()
        x = P.reshape(-1)
        if k < 8:
            err = np.abs(x - fx["cubes_poses"][k + 1]).max()
            assert err <= POSE_ATOL, (k, err)
        assert ctx.detect_intersections(x) == 0, k
    assert ctx.compute_min_distance(x, SF.DHAT) > 0
    assert fx["cubes_min_distance"][-1] > 0
    # resting heights: three layers of nine cubes on the plane at the end (a
    # perturbed oracle run settles to the same heights within 1e-6)
    dyn = np.array([b.type == 2 for b in sc.bodies])
    y_g = P[dyn, 1]
    y_o = fx["cubes_poses"][-1].reshape(-1, 6)[dyn, 1]
    assert np.abs(np.sort(y_g) - np.sort(y_o)).max() < 1e-4


def test_detect_intersections_matches_oracle(oracle):
    """Crossing (edge, face) pairs at intersecting poses (every cube sunk
    1 cm, one cube sunk 30 cm) and at the resting contact, GPU and oracle."""
    import rigc
    from conftest import contact_poses

    import make_step_fixtures as SF

    sc = SF.cubes_scene()
    o = oracle.OracleScene(sc)
    ctx = rigc.Context(sc)
    x = contact_poses(sc).reshape(-1, 6)
    dyn = np.array([b.type == 2 for b in sc.bodies])
    sunk = x.copy()
    sunk[dyn, 1] -= 0.01
    deep = x.copy()
    deep[np.where(dyn)[0][0], 1] -= 0.3
    counts = []
    for y in (x, sunk, deep):
        n_o = o.detect_intersections(y.reshape(-1))
        assert ctx.detect_intersections(y.reshape(-1)) == n_o
        counts.append(n_o)
    assert counts[0] == 0 and counts[1] > 0 and counts[2] > 0


@pytest.mark.parametrize("case", ["pair", "pile"])
def test_friction_steps_match_oracle(case):
    """Time steps with friction (mu 0.5, one lagged friction iteration per
    step): two cubes sliding into each other on the plane (10 steps) and 8
    icospheres in a contact pile (2 steps), poses within 1e-8 of the
    oracle's and intersection-free."""
    import rigc

    import make_step_fixtures as SF

    if case == "pair":
        sc, x0, steps = SF.pair_scene(), None, SF.PAIR_STEPS
    else:
        (sc, x0), steps = SF.pile_scene(), SF.PILE_STEPS
    fx = _fixture(case, sc, sc.poses() if x0 is None else x0)
    ctx = rigc.Context(sc)
    ctx.sim_init(SF.H, SF.G, SF.DHAT, coefficient_friction=SF.MU, poses=x0)
    for k in range(steps):
        ctx.sim_step(1)
        P, V, Q, kappa = ctx.sim_state()
        err = np.abs(P.reshape(-1) - fx[case + "_poses"][k + 1]).max()
        assert err <= POSE_ATOL, (k, err)
        assert kappa == pytest.approx(float(fx[case + "_kappa"][k]), rel=1e-9)
        assert ctx.detect_intersections(P.reshape(-1)) == 0
