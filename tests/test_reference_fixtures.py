"""The reference's own CCD test data, packed by
tests/golden/make_reference_fixtures.py (see its header for the sources):
the oracle must reproduce the stored results exactly.

* 403 edge-edge / face-vertex queries (tests/data/{wrecking-ball,kinematic}/
  and tests/data/ccd-test-*.json of the reference, as read by
  tests/ccd/test_rigid_body_time_of_impact.cpp:597-853): time of impact and
  status per query;
* the 575-body wrecking-ball scene (tests/data/large-rb-hashgrid/): the
  continuous candidate set.
"""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def queries():
    return np.load(os.path.join(GOLD, "reference_ccd_queries.npz"))


def scene_fixture():
    return np.load(os.path.join(GOLD, "wrecking_ball_scene.npz"))


def test_reference_queries_oracle(oracle):
    import make_reference_fixtures as M

    q = queries()
    assert len(q["kind"]) == 403
    for k, V, P, toi, st in zip(q["kind"], q["vertices"], q["poses"], q["toi_oracle"],
                                q["status_oracle"]):
        t, s = M.oracle_toi(int(k), V, P)
        assert (t == toi or (np.isinf(t) and np.isinf(toi))) and s == st
    # the queries whose bodies touch at t = 0 end at the budget with t = 0
    capped = q["status_oracle"] != 0
    assert capped.sum() == 6 and np.all(q["toi_oracle"][capped] == 0.0)


def test_wrecking_ball_candidates_oracle(oracle):
    import make_reference_fixtures as M

    d = scene_fixture()
    sc = M.scene_from_fixture(d)
    o = oracle.OracleScene(sc)
    ee, fv = o.detect_candidates(d["pose_t0"].reshape(-1), d["pose_t1"].reshape(-1), True, 0.0)
    assert len(ee) == int(d["num_ee"]) and len(fv) == int(d["num_fv"])
    assert M.candidates_digest(ee, fv) == str(d["candidates_sha256"])
