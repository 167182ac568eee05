"""Pack the reference's own CCD test data into small fixtures for this repo.

Run in a checkout that has the rigid-ipc source tree (read only):

    python tests/golden/make_reference_fixtures.py /path/to/rigid-ipc

Inputs (the reference's test data, used by
tests/ccd/test_rigid_body_time_of_impact.cpp:597-853 and, for the scene,
tests/ccd/test_rigid_body_hash_grid.cpp:104-140):
  * tests/data/wrecking-ball/ccd-test-*.json, tests/data/kinematic/ccd-test-*.json,
    tests/data/ccd-test-*.json: one edge-edge or face-vertex query each, two
    bodies whose rest vertices are used as given (create_body cancels the
    inertial frame) and their poses at t0 and t1;
  * tests/data/large-rb-hashgrid/large-rb-hashgrid-000.json: a 575-body
    wrecking-ball scene with poses at t0 and t1.

Outputs (tests/golden/):
  * reference_ccd_queries.npz: kind (0 edge-edge, 1 face-vertex), vertices
    (4 x 3: EE edge0 v0 v1, edge1 v0 v1; FV face v0 v1 v2, vertex), poses
    (2 x 2 x 6: [body][t0, t1][p, theta]; body 0 = edge0 / face, body 1 =
    edge1 / vertex), source file names, and the oracle's time of impact and
    status of each query at the reference's default tolerance (1e-4) with a
    budget of 2^16 boxes per query (the queries whose bodies touch at t = 0
    would search forever without one: the reference has no cap);
  * wrecking_ball_scene.npz: the scene's distinct meshes, the mesh of each
    body, the poses at t0 and t1, and the oracle's results on it: the
    continuous candidate set (inflation 0; counts and a SHA-256 of the
    sorted (edge, edge) then (face, vertex) int32 pairs, checked equal to a
    brute-force box sweep) and every candidate's time of impact (tolerance
    1e-4, 2^16 boxes per candidate, no cross-candidate pruning), stored as
    the indices and values of the finite ones.

Edge-vertex queries ("ev", 2D in the reference) are skipped, as the
reference's test skips them.
"""
from __future__ import annotations

import glob
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _pose(j):
    return np.array(list(j["position"]) + list(j["rotation"]), np.float64)


def load_queries(ref):
    files = []
    for sub in ("wrecking-ball", "kinematic", ""):
        files += sorted(glob.glob(os.path.join(ref, "tests", "data", sub, "ccd-test-*.json")))
    kinds, verts, poses, names = [], [], [], []
    for f in files:
        with open(f) as fh:
            j = json.load(fh)
        t = j["type"]
        if t == "ee":
            V = [j["edge0"]["vertex0"], j["edge0"]["vertex1"], j["edge1"]["vertex0"],
                 j["edge1"]["vertex1"]]
            P = [[_pose(j["edge0"]["pose_t0"]), _pose(j["edge0"]["pose_t1"])],
                 [_pose(j["edge1"]["pose_t0"]), _pose(j["edge1"]["pose_t1"])]]
            kinds.append(0)
        elif t == "fv":
            V = [j["face"]["vertex0"], j["face"]["vertex1"], j["face"]["vertex2"],
                 j["vertex"]["vertex"]]
            P = [[_pose(j["face"]["pose_t0"]), _pose(j["face"]["pose_t1"])],
                 [_pose(j["vertex"]["pose_t0"]), _pose(j["vertex"]["pose_t1"])]]
            kinds.append(1)
        else:
            continue
        verts.append(np.array(V, np.float64))
        poses.append(np.array(P, np.float64))
        names.append(os.path.relpath(f, os.path.join(ref, "tests", "data")))
    return np.array(kinds, np.int32), np.array(verts), np.array(poses), np.array(names)


def query_scene(kind, V):
    """Two raw bodies of one query (scene body 0 = edge0 / face)."""
    from rigc import scene as S

    if kind == 0:
        a = S.raw_body(V[0:2], edges=[[0, 1]], group_id=0)
        b = S.raw_body(V[2:4], edges=[[0, 1]], group_id=1)
    else:
        a = S.raw_body(V[0:3], faces=[[0, 1, 2]], group_id=0)
        b = S.raw_body(V[3:4], edges=np.zeros((0, 2), np.int32), group_id=1)
    return S.Scene(bodies=[a, b])


BUDGET = 1 << 16  # boxes per query; the queries at t = 0 never finish without one


def oracle_toi(kind, V, P, tol=1e-4):
    import oracle as O

    sc = query_scene(kind, V)
    o = O.OracleScene(sc)
    x0 = np.concatenate([P[0, 0], P[1, 0]])
    x1 = np.concatenate([P[0, 1], P[1, 1]])
    if kind == 0:
        ee = np.array([[0, 1]], np.int32)
        fv = np.zeros((0, 2), np.int32)
    else:
        ee = np.zeros((0, 2), np.int32)
        fv = np.array([[0, 3]], np.int32)
    t, per, _, status = o.earliest_toi(x0, x1, ee, fv, tol=tol, per_candidate=True,
                                       max_boxes=BUDGET, with_status=True)
    return per[0], status


def load_scene(ref):
    path = os.path.join(ref, "tests", "data", "large-rb-hashgrid", "large-rb-hashgrid-000.json")
    with open(path) as fh:
        bodies = json.load(fh)["bodies"]
    meshes, mesh_of = [], []
    for b in bodies:
        V = np.array(b["vertices"], np.float64)
        E = np.array(b["edges"], np.int32)
        F = np.array(b["faces"], np.int32)
        for k, (V2, E2, F2) in enumerate(meshes):
            if V2.shape == V.shape and np.array_equal(V2, V) and np.array_equal(E2, E) \
                    and np.array_equal(F2, F):
                mesh_of.append(k)
                break
        else:
            meshes.append((V, E, F))
            mesh_of.append(len(meshes) - 1)
    out = {"mesh_of": np.array(mesh_of, np.int32),
           "pose_t0": np.array([_pose(b["pose_t0"]) for b in bodies]),
           "pose_t1": np.array([_pose(b["pose_t1"]) for b in bodies]),
           "num_meshes": np.int32(len(meshes))}
    for k, (V, E, F) in enumerate(meshes):
        out[f"V{k}"] = V
        out[f"E{k}"] = E
        out[f"F{k}"] = F
    return out


def scene_from_fixture(d):
    from rigc import scene as S

    bodies = []
    for i, m in enumerate(d["mesh_of"]):
        bodies.append(S.raw_body(d[f"V{m}"], edges=d[f"E{m}"], faces=d[f"F{m}"], group_id=i))
    return S.Scene(bodies=bodies)


def candidates_digest(ee, fv):
    import hashlib

    h = hashlib.sha256()
    h.update(np.ascontiguousarray(ee, np.int32).tobytes())
    h.update(np.ascontiguousarray(fv, np.int32).tobytes())
    return h.hexdigest()


def scene_results(d, nthreads):
    import oracle as O

    sc = scene_from_fixture(d)
    o = O.OracleScene(sc)
    x0 = d["pose_t0"].reshape(-1)
    x1 = d["pose_t1"].reshape(-1)
    ee, fv = o.detect_candidates(x0, x1, True, 0.0)
    eb, fb = o.detect_candidates(x0, x1, True, 0.0, brute=True)
    assert np.array_equal(ee, eb) and np.array_equal(fv, fb)
    toi, per, _, status = o.earliest_toi(x0, x1, ee, fv, tol=1e-4, nthreads=nthreads,
                                         per_candidate=True, max_boxes=BUDGET, with_status=True)
    idx = np.flatnonzero(np.isfinite(per)).astype(np.int32)
    return {"num_ee": np.int64(len(ee)), "num_fv": np.int64(len(fv)),
            "candidates_sha256": np.array(candidates_digest(ee, fv)),
            "toi_idx": idx, "toi_val": per[idx], "toi_min": np.float64(toi),
            "status_oracle": np.int32(status), "budget": np.int64(BUDGET)}


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RIGID_IPC_SOURCE", "")
    if not ref or not os.path.isdir(os.path.join(ref, "tests", "data")):
        sys.exit("usage: make_reference_fixtures.py <rigid-ipc source tree>")
    sys.path[:0] = [os.path.join(ROOT, "rigid-ipc_gb300"), os.path.join(ROOT, "oracle")]
    kinds, verts, poses, names = load_queries(ref)
    res = [oracle_toi(k, V, P) for k, V, P in zip(kinds, verts, poses)]
    tois = np.array([r[0] for r in res])
    status = np.array([r[1] for r in res], np.int32)
    np.savez_compressed(os.path.join(HERE, "reference_ccd_queries.npz"), kind=kinds, vertices=verts,
                        poses=poses, name=names, toi_oracle=tois, status_oracle=status,
                        budget=np.int64(BUDGET))
    print(f"{len(kinds)} queries, {int(np.isfinite(tois).sum())} with an impact, "
          f"{int((status != 0).sum())} at the box budget")
    scene = load_scene(ref)
    scene.update(scene_results(scene, os.cpu_count() or 1))
    np.savez_compressed(os.path.join(HERE, "wrecking_ball_scene.npz"), **scene)
    print(f"scene written: {int(scene['num_ee'])} + {int(scene['num_fv'])} candidates, "
          f"{len(scene['toi_idx'])} with an impact, status {int(scene['status_oracle'])}")


if __name__ == "__main__":
    main()
