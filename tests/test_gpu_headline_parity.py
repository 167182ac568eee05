"""Parity at the benchmark's headline workload, at full size.

The 1000-icosphere contact pile that bench.py times (bench.make_workload(1000,
0): 632,682 continuous and 109,007 discrete candidates): every output of the
narrow-phase pass against the oracle run on the same inputs in this process,
and the oracle against the committed fixture tests/golden/
headline_pile_1000.npz (made by make_headline_fixture.py) wherever this
machine builds the same scene bit for bit.

Bars: candidate sets, the earliest time of impact, per-candidate times of
impact and the constraint set bit-exact; barrier energy and gradient 1e-10
relative; assembled Hessian blocks 1e-9 relative (Frobenius, per block row).
"""
import os

import numpy as np
import pytest

import make_headline_fixture as F

pytestmark = pytest.mark.gpu

ENERGY_RTOL = 1e-10
GRAD_RTOL = 1e-10
HESS_RTOL = 1e-9
FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                       "headline_pile_1000.npz")


@pytest.fixture(scope="module")
def pile():
    import rigc

    sc, x0, x1 = F.workload()
    r = F.oracle_results(sc, x0, x1)
    ctx = rigc.Context(sc)
    return sc, x0, x1, r, ctx


def test_oracle_matches_fixture(pile):
    sc, x0, x1, r, _ = pile
    fx = np.load(FIXTURE)
    if F.digest(sc.rest_vertices, x0, x1) != str(fx["input_digest"]):
        pytest.skip("this machine builds a different pile (floating-point set-up differs)")
    assert F.digest(r["ee"]) == str(fx["ee_digest"]) and F.digest(r["fv"]) == str(fx["fv_digest"])
    assert F.digest(r["ee_d"]) == str(fx["ee_d_digest"])
    assert F.digest(r["fv_d"]) == str(fx["fv_d_digest"])
    assert r["toi"] == float(fx["toi"])
    assert np.array_equal(r["sample_toi"], fx["sample_toi"])
    assert np.array_equal(r["cs"].types, fx["cs_types"])
    assert r["energy"] == float(fx["energy"]) and np.array_equal(r["grad"], fx["grad"])


def test_fixture_sizes():
    fx = np.load(FIXTURE)
    assert int(fx["n_ee"]) + int(fx["n_fv"]) == 632682
    assert int(fx["n_ee_d"]) + int(fx["n_fv_d"]) == 109007


def test_continuous_candidates(pile):
    sc, x0, x1, r, ctx = pile
    ee, fv = ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    assert len(ee) + len(fv) == 632682
    assert np.array_equal(ee, r["ee"]) and np.array_equal(fv, r["fv"])


def test_discrete_candidates(pile):
    sc, x0, x1, r, ctx = pile
    ee, fv = ctx.detect_collision_candidates_rigid(x0, x0, False, F.DHAT / 2)
    assert np.array_equal(ee, r["ee_d"]) and np.array_equal(fv, r["fv_d"])


def test_earliest_toi(pile):
    sc, x0, x1, r, ctx = pile
    ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    assert ctx.earliest_toi(x0, x1, prune=True) == r["toi"]
    assert ctx.compute_earliest_toi(x0, x1) == r["toi"]


def test_per_candidate_toi_sample(pile):
    sc, x0, x1, r, ctx = pile
    ee_s, fv_s = r["ee"][r["sample_ee"]], r["fv"][r["sample_fv"]]
    assert len(ee_s) + len(fv_s) == F.SAMPLE
    ctx.set_candidates(ee_s, fv_s)
    toi, per, st = ctx.earliest_toi(x0, x1, prune=False, per_candidate=True)
    assert st == 0
    assert np.array_equal(per, r["sample_toi"])
    assert toi == r["sample_toi"].min()


def test_constraint_set_and_barrier(pile):
    from test_gpu_parity import _canon_constraints

    sc, x0, x1, r, ctx = pile
    import oracle as O

    cs_o = r["cs"]
    cs = ctx.construct_constraint_set(x0, F.DHAT)
    assert len(cs_o) == 133
    a = _canon_constraints(cs_o.types, cs_o.verts, cs_o.prims, cs_o.bodies, cs_o.weight, cs_o.eps)
    b = _canon_constraints(cs["type"], cs["verts"], cs["prims"], cs["bodies"], cs["weight"],
                           cs["eps"])
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    e_g, g_g, (rp_g, col_g, val_g) = ctx.compute_barrier_term(x0, F.DHAT)
    e_o, g_o, (rp_o, col_o, val_o) = O.OracleScene(sc).barrier_term(x0, cs_o, F.DHAT)
    assert abs(e_g - e_o) <= ENERGY_RTOL * abs(e_o)
    assert np.abs(g_g - g_o).max() <= GRAD_RTOL * np.abs(g_o).max()
    assert np.array_equal(rp_g, rp_o) and np.array_equal(col_g, col_o)
    for row in range(len(rp_o) - 1):
        blk_o = val_o[rp_o[row]:rp_o[row + 1]]
        blk_g = val_g[rp_o[row]:rp_o[row + 1]]
        if blk_o.size:
            assert np.linalg.norm(blk_g - blk_o) <= HESS_RTOL * np.linalg.norm(blk_o)


@pytest.mark.parametrize("warp", [1, 2, 5])
def test_earliest_toi_time_windows(pile, warp):
    """The pruned earliest time of impact with the CCD's time windows (first
    window 2^-k, doubled each launch; k = 0: none) is the oracle's bit for
    bit whatever the window, and the windows search fewer boxes than one
    launch under the running minimum alone."""
    sc, x0, x1, r, ctx = pile
    ctx.detect_collision_candidates_rigid(x0, x1, True, 0.0)
    ctx.set_tune(ccd_warp=warp)
    boxes = {}
    try:
        for k in (0, 2, 7, 12):
            ctx.set_ccd_window(k)
            assert ctx.earliest_toi(x0, x1, prune=True) == r["toi"], k
            boxes[k] = ctx.stats()["ccd_boxes"]
    finally:
        ctx.set_ccd_window(-1)
        ctx.set_tune()
    assert boxes[7] < boxes[0]
