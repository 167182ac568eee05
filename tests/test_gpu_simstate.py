"""Simulation runs with the reference's results file (SimState): the state
sequence written after every step, checkpoints, and a run resumed from a
checkpoint that continues exactly as the run that was never stopped."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_results_file_and_resume(tmp_path):
    from rigc import scene as S
    from rigc.simstate import SimState

    spec = S.spec_cubes(0)
    spec["max_time"] = 0.12  # 12 steps
    out = str(tmp_path / "run.json")
    a = SimState(spec).run(out=out, checkpoint_every=5)
    with open(out) as f:
        res = json.load(f)
    seq = res["animation"]["state_sequence"]
    assert len(seq) == 13 and res["args"]["timestep"] == 0.01
    assert len(seq[-1]["rigid_bodies"]) == a.scene.num_bodies
    for k in ("step_timings", "solver_iterations", "num_contacts", "step_minimum_distances"):
        assert len(res["stats"][k]) == 12
    assert res["stats"]["intersecting_steps"] == []
    chk = str(tmp_path / "run-chkpt00010.json")
    with open(chk) as f:
        assert len(json.load(f)["animation"]["state_sequence"]) == 11
    # resume at step 10 and run the last 2 steps: the same states, bit for bit
    b = SimState.load(chk).run(steps=2)
    assert b.num_steps == 12
    for k in (11, 12):
        for ra, rb in zip(a.state_sequence[k]["rigid_bodies"], b.state_sequence[k]["rigid_bodies"]):
            assert ra["position"] == rb["position"] and ra["rotation"] == rb["rotation"]
            assert np.array_equal(ra["Qdot"], rb["Qdot"])
