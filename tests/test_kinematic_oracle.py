"""Kinematic bodies (the augmented Lagrangian of
DistanceBarrierRBProblem::compute_augmented_lagrangian,
src/problems/distance_barrier_rb_problem.cpp:946-1109) in the oracle's time
step: a kinematic body follows x0 + h v each step; pushing a dynamic body it
still meets its target to the reference's tolerance (progress >= 0.999)."""
import numpy as np

H = 0.01
G = (0.0, -9.81, 0.0)


def paddle_scene(push=True):
    from rigc import meshes, scene as S

    V, F = meshes.cube()
    bodies = [S.make_body(V, F, position=(0.0, 0.6, 0.0), linear_velocity=(2.0, 0.0, 0.0),
                          angular_velocity_deg=(0.0, 30.0, 0.0), body_type="kinematic")]
    if push:
        bodies.append(S.make_body(V, F, position=(1.03, 0.5008, 0.0)))
    Vp, Fp = meshes.plane(20.0)
    bodies.append(S.make_body(Vp, Fp, body_type="static"))
    S.assign_group_ids(bodies)
    return S.Scene(bodies=bodies)


def test_kinematic_body_follows_its_velocity(oracle):
    sc = paddle_scene(push=False)
    sim = oracle.OracleSim(sc, h=H, gravity=G, dhat=1e-3)
    x = sc.poses().reshape(-1, 6)[0].copy()
    v = sc.velocities().reshape(-1, 6)[0]
    for _ in range(3):
        prev = sim.pose[:6].copy()
        sim.step()
        x = x + H * v
        # the linear target is met exactly (a quadratic), the rotation to the
        # reference's progress tolerance (0.1 % of the step)
        assert np.abs(sim.pose[:3] - x[:3]).max() <= 1e-12
        assert np.linalg.norm(sim.pose[3:6] - (prev[3:6] + H * v[3:])) <= 1e-3 * H * np.linalg.norm(v[3:])
        x[3:] = sim.pose[3:6]


def test_kinematic_body_pushes_dynamic_one(oracle):
    sc = paddle_scene()
    sim = oracle.OracleSim(sc, h=H, gravity=G, dhat=1e-3)
    x0 = sc.poses().reshape(-1, 6).copy()
    v = sc.velocities().reshape(-1, 6)[0]
    o = oracle.OracleScene(sc)
    for k in range(4):
        prev = sim.pose.reshape(-1, 6)[0].copy()
        sim.step()
        P = sim.pose.reshape(-1, 6)
        # the kinematic body meets its target x0 + h v within 0.1% of the step
        target = prev + H * v
        assert np.linalg.norm(P[0, :3] - target[:3]) <= 1e-3 * np.linalg.norm(H * v[:3]) + 1e-12
        ee, fv = o.detect_candidates(sim.pose, continuous=False, inflation=5e-4)
        cs = o.constraint_set(sim.pose, ee, fv, 1e-3)
        if len(cs):
            e, _, _ = o.local_terms(sim.pose, cs, 1e-3)
            assert np.all(np.isfinite(e))
    # the dynamic cube was pushed along +x
    assert P[1, 0] - x0[1, 0] > 1e-3


def scheduled_scene(max_time=0.05, n_poses=3):
    """A kinematic cube with a pose list (JSON kinematic_poses) and a
    kinematic_max_time, a dynamic cube in its way, a static plane."""
    from rigc import scene as S

    poses = [{"position": [0.2 + 0.1 * (k + 1), 0.6, 0.0], "rotation": [0.0, 0.05 * (k + 1), 0.0]}
             for k in range(n_poses)]
    spec = {"timestep": H, "rigid_body_problem": {"gravity": list(G), "rigid_bodies": [
        {"mesh": "plane", "type": "static", "scale": 20.0},
        {"mesh": "cube", "type": "kinematic", "position": [0.2, 0.6, 0.0],
         "linear_velocity": [0.5, 0.0, 0.0], "kinematic_max_time": max_time,
         "kinematic_poses": poses},
        {"mesh": "cube", "position": [1.27, 0.5008, 0.0]}]}}
    return S.scene_from_json(spec)


def test_scene_reads_kinematic_schedule():
    """read_rb_scene.cpp:94-101,233-245: the pose list as given, a negative
    max time as no limit."""
    from rigc import scene as S

    sc = scheduled_scene()
    b = sc.bodies[1]
    assert b.kinematic_max_time == 0.05 and len(b.kinematic_poses) == 3
    assert np.array_equal(b.kinematic_poses[1], [0.4, 0.6, 0.0, 0.0, 0.1, 0.0])
    spec = {"rigid_body_problem": {"rigid_bodies": [
        {"mesh": "cube", "type": "kinematic", "kinematic_max_time": -1}]}}
    assert S.scene_from_json(spec).bodies[0].kinematic_max_time == np.inf


def test_kinematic_schedule(oracle):
    """The body is driven to each listed pose in turn (positions to the
    augmented Lagrangian's progress tolerance), then by its velocity; once
    kinematic_max_time has run out it is static: type 0, every dof fixed,
    velocity zero, pose unchanged from then on (init_augmented_lagrangian and
    step_kinematic_bodies, distance_barrier_rb_problem.cpp:190-251)."""
    sc = scheduled_scene()
    sim = oracle.OracleSim(sc, h=H, gravity=G, dhat=1e-3)
    targets = [np.asarray(q) for q in sc.bodies[1].kinematic_poses]
    for k in range(3):
        prev = sim.pose[6:12].copy()
        sim.step()
        P = sim.pose[6:12]
        step = np.linalg.norm(targets[k][:3] - prev[:3])
        assert np.linalg.norm(P[:3] - targets[k][:3]) <= 1e-3 * step + 1e-12
        assert sim.type[1] == 1
    # the list used up: x0 + h v (v the initial 0.5 m/s along x)
    prev = sim.pose[6:12].copy()
    sim.step()
    assert abs(sim.pose[6] - (prev[0] + H * 0.5)) <= 1e-3 * H * 0.5 + 1e-12
    # 0.05 s run out after five steps: static from the sixth step's start
    sim.step()
    sim.step()
    assert sim.type[1] == 0 and np.all(sim.fixed[6:12] == 1) and np.all(sim.vel[6:12] == 0)
    frozen = sim.pose[6:12].copy()
    sim.step()
    assert np.array_equal(sim.pose[6:12], frozen)
