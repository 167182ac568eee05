"""Parity of the CUDA friction path (through the C ABI) with the CPU oracle.

Bars: closest points and tangent bases bit-exact (the set-up follows the
oracle's round-to-nearest operation order); normal force magnitudes within
1e-10 relative; energy and gradient within 1e-10, Hessians within 1e-9
relative (Frobenius, per local 12x12 or per assembled block).
"""
import numpy as np
import pytest

from test_friction_oracle import DHAT, EPSVH, KAPPA, MU, _friction_setup, point_on_triangle

pytestmark = pytest.mark.gpu

RTOL = 1e-10
HESS_RTOL = 1e-9


def _gpu_ctx(scene, cs, x0):
    import rigc

    ctx = rigc.Context(scene)
    ctx.set_constraints(cs.types, cs.verts, cs.prims, cs.bodies, cs.weight, cs.eps)
    n = ctx.friction_setup(x0, DHAT, KAPPA, MU)
    assert n == len(cs)
    return ctx


def test_friction_setup_parity(oracle, cube_scene, cube_contact):
    o, x0, cs, fc, x = _friction_setup(oracle, cube_scene, cube_contact, 1)
    ctx = _gpu_ctx(cube_scene, cs, x0)
    f = ctx.friction_constraints()
    lam, params, T = fc
    assert np.array_equal(f["type"], cs.types)
    assert f["mu"] == MU
    # lambda goes through log(), whose last bits differ between libraries
    assert np.abs(f["lambda"] - lam).max() <= RTOL * np.abs(lam).max()
    # closest points and bases follow the oracle's round-to-nearest operation
    # order (nearly parallel edges make the closest points ill-conditioned,
    # so only bit equality is a meaningful bar for them)
    assert np.array_equal(f["closest"], params)
    assert np.array_equal(f["basis"], T)


@pytest.mark.parametrize("project", [False, True])
def test_friction_local_terms_parity(oracle, cube_scene, cube_contact, project):
    o, x0, cs, fc, x = _friction_setup(oracle, cube_scene, cube_contact, 2)
    ctx = _gpu_ctx(cube_scene, cs, x0)
    # the GPU's own setup (bases may differ by rounding; the potential does not)
    f = ctx.friction_constraints()
    fc_g = (f["lambda"], f["closest"], f["basis"])
    e_o, g_o, H_o = o.friction_local_terms(x, x0, cs, fc_g, MU, EPSVH, project=project)
    e_g, g_g, H_g = ctx.friction_local_terms(x, len(cs), EPSVH, project=project)
    gs = np.abs(g_o).max()
    for i in range(len(cs)):
        assert abs(e_g[i] - e_o[i]) <= RTOL * max(abs(e_o[i]), 1e-300)
        assert np.abs(g_g[i] - g_o[i]).max() <= RTOL * max(np.abs(g_o[i]).max(), 1e-6 * gs)
        nh = np.linalg.norm(H_o[i])
        assert np.linalg.norm(H_g[i] - H_o[i]) <= HESS_RTOL * max(nh, 1e-300)


def test_friction_term_assembled(oracle, cube_scene, cube_contact):
    o, x0, cs, fc, x = _friction_setup(oracle, cube_scene, cube_contact, 3)
    ctx = _gpu_ctx(cube_scene, cs, x0)
    f = ctx.friction_constraints()
    fc_g = (f["lambda"], f["closest"], f["basis"])
    e_o, g_o, (rp_o, col_o, val_o) = o.friction_term(x, x0, cs, fc_g, MU, EPSVH)
    e_g, g_g, (rp_g, col_g, val_g) = ctx.compute_friction_term(x, EPSVH)
    assert abs(e_g - e_o) <= RTOL * abs(e_o)
    assert np.abs(g_g - g_o).max() <= RTOL * np.abs(g_o).max()
    assert np.array_equal(rp_g, rp_o) and np.array_equal(col_g, col_o)
    for r in range(len(rp_o) - 1):
        blk_o = val_o[rp_o[r]:rp_o[r + 1]]
        blk_g = val_g[rp_o[r]:rp_o[r + 1]]
        if blk_o.size:
            assert np.linalg.norm(blk_g - blk_o) <= HESS_RTOL * max(np.linalg.norm(blk_o), 1e-300)
    # a barrier term computed in between leaves the friction outputs intact
    ctx.compute_barrier_term(x0, DHAT)
    e2, g2, _ = ctx.compute_friction_term(x, EPSVH, hess=False)
    assert e2 == e_g and np.array_equal(g2, g_g)


def test_friction_known_answer_gpu(oracle):
    gap = 4e-4
    sc = point_on_triangle(gap)
    o = oracle.OracleScene(sc)
    x0 = np.zeros(12)
    ee, fv = o.detect_candidates(x0, continuous=False, inflation=DHAT / 2)
    cs = o.constraint_set(x0, ee, fv, DHAT)
    ctx = _gpu_ctx(sc, cs, x0)
    x = x0.copy()
    x[6] = 3e-4
    lam = ctx.friction_constraints()["lambda"]
    e, g, _ = ctx.compute_friction_term(x, EPSVH)
    assert e == pytest.approx(MU * lam.sum() * 3e-4, rel=1e-12)
    assert g[6] > 0 and g[0] == pytest.approx(-g[6], rel=1e-12)


def test_friction_empty(cube_scene):
    import rigc

    ctx = rigc.Context(cube_scene)
    empty = np.zeros(0, np.int32)
    ctx.set_constraints(empty, np.zeros((0, 4), np.int32), np.zeros((0, 2), np.int32),
                        np.zeros((0, 2), np.int32), np.zeros(0), np.zeros(0))
    assert ctx.friction_setup(cube_scene.poses(), DHAT, KAPPA, MU) == 0
    e, g, (rp, col, val) = ctx.compute_friction_term(cube_scene.poses(), EPSVH)
    assert e == 0.0 and not g.any() and not rp.any() and len(col) == 0
