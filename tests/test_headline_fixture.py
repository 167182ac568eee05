"""The oracle on the benchmark's headline workload against its committed
fixture (tests/golden/headline_pile_1000.npz, made by
make_headline_fixture.py), when this machine builds the same pile."""
import os

import numpy as np
import pytest

import make_headline_fixture as F

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                       "headline_pile_1000.npz")


def test_oracle_reproduces_headline_fixture():
    sc, x0, x1 = F.workload()
    fx = np.load(FIXTURE)
    if F.digest(sc.rest_vertices, x0, x1) != str(fx["input_digest"]):
        pytest.skip("this machine builds a different pile (floating-point set-up differs)")
    r = F.oracle_results(sc, x0, x1)
    assert F.digest(r["ee"]) == str(fx["ee_digest"]) and F.digest(r["fv"]) == str(fx["fv_digest"])
    assert F.digest(r["ee_d"]) == str(fx["ee_d_digest"])
    assert F.digest(r["fv_d"]) == str(fx["fv_d_digest"])
    assert r["toi"] == float(fx["toi"])
    assert np.array_equal(r["sample_toi"], fx["sample_toi"])
    assert np.array_equal(r["cs"].types, fx["cs_types"])
    assert np.array_equal(r["cs"].verts, fx["cs_verts"])
    assert r["energy"] == float(fx["energy"]) and np.array_equal(r["grad"], fx["grad"])
