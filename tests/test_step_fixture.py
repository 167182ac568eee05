"""The oracle's time step against its committed trajectories
(tests/golden/step_trajectories.npz, made by make_step_fixtures.py): the
first steps of the 27-cube lattice and the sliding cube pair with friction,
bit for bit, when this machine builds the same scenes."""
import os

import numpy as np
import pytest

import make_step_fixtures as SF

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                       "step_trajectories.npz")


@pytest.mark.parametrize("case", ["cubes", "pair"])
def test_oracle_reproduces_step_fixture(case):
    sc = SF.cubes_scene() if case == "cubes" else SF.pair_scene()
    fx = np.load(FIXTURE)
    if SF.inputs_digest(sc, sc.poses()) != str(fx[case + "_digest"]):
        pytest.skip("this machine builds a different scene (floating-point set-up differs)")
    steps = 3 if case == "cubes" else SF.PAIR_STEPS
    poses, kappa, _, _ = SF.run(sc, steps, mu=0.0 if case == "cubes" else SF.MU)
    assert np.array_equal(poses, fx[case + "_poses"][:steps + 1])
    assert np.array_equal(kappa, fx[case + "_kappa"][:steps])
