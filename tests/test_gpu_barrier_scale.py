"""The barrier terms at scale: the contact-heavy slab stacks that bench.py
times for the barrier (4 x 4 columns of 2 tessellated slabs resting 0.3 mm
apart, some 1.6 x 10^5 constraints), against the oracle.

Bars: discrete candidate set and constraint set bit-exact; barrier energy and
gradient 1e-10 relative; assembled Hessian blocks 1e-9 relative (Frobenius,
per block row); the per-constraint 12x12 Hessians (raw and PSD-projected)
1e-9 on a seeded sample of 2,000 constraints.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ENERGY_RTOL = 1e-10
GRAD_RTOL = 1e-10
HESS_RTOL = 1e-9
DHAT = 1e-3


@pytest.fixture(scope="module")
def slabs():
    import oracle as O
    import rigc
    from rigc import scene as S

    O.build()
    sc = S.scene_from_json(S.spec_slab_stacks(0, nx=4, nz=4))
    x = sc.poses()
    o = O.OracleScene(sc)
    ee, fv = o.detect_candidates(x, continuous=False, inflation=DHAT / 2)
    cs = o.constraint_set(x, ee, fv, DHAT)
    return sc, x, o, ee, fv, cs, rigc.Context(sc)


def test_slab_candidates_and_constraints(slabs):
    from test_gpu_parity import _canon_constraints

    sc, x, o, ee, fv, cs_o, ctx = slabs
    assert len(cs_o) > 100_000
    ee_g, fv_g = ctx.detect_collision_candidates_rigid(x, x, False, DHAT / 2)
    assert np.array_equal(ee_g, ee) and np.array_equal(fv_g, fv)
    cs = ctx.construct_constraint_set(x, DHAT)
    a = _canon_constraints(cs_o.types, cs_o.verts, cs_o.prims, cs_o.bodies, cs_o.weight, cs_o.eps)
    b = _canon_constraints(cs["type"], cs["verts"], cs["prims"], cs["bodies"], cs["weight"],
                           cs["eps"])
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_slab_barrier_term(slabs):
    sc, x, o, ee, fv, cs_o, ctx = slabs
    ctx.construct_constraint_set(x, DHAT)
    e_g, g_g, (rp_g, col_g, val_g) = ctx.compute_barrier_term(x, DHAT)
    e_o, g_o, (rp_o, col_o, val_o) = o.barrier_term(x, cs_o, DHAT)
    assert abs(e_g - e_o) <= ENERGY_RTOL * abs(e_o)
    assert np.abs(g_g - g_o).max() <= GRAD_RTOL * np.abs(g_o).max()
    assert np.array_equal(rp_g, rp_o) and np.array_equal(col_g, col_o)
    for r in range(len(rp_o) - 1):
        blk_o = val_o[rp_o[r]:rp_o[r + 1]]
        blk_g = val_g[rp_o[r]:rp_o[r + 1]]
        if blk_o.size:
            assert np.linalg.norm(blk_g - blk_o) <= HESS_RTOL * np.linalg.norm(blk_o)


@pytest.mark.parametrize("project", [False, True])
def test_slab_local_terms_sample(slabs, project):
    import oracle as O

    sc, x, o, ee, fv, cs_o, ctx = slabs
    rng = np.random.default_rng(5)
    sel = np.sort(rng.choice(len(cs_o), size=2000, replace=False))
    sub = O.Constraints(cs_o.types[sel], cs_o.verts[sel], cs_o.prims[sel], cs_o.bodies[sel],
                        cs_o.weight[sel], cs_o.eps[sel])
    ctx.set_constraints(sub.types, sub.verts, sub.prims, sub.bodies, sub.weight, sub.eps)
    e_g, g_g, H_g = ctx.barrier_local_terms(x, len(sub), DHAT, project=project)
    e_o, g_o, H_o = o.local_terms(x, sub, DHAT, project=project)
    assert np.all(np.abs(e_g - e_o) <= ENERGY_RTOL * np.abs(e_o))
    gs = np.maximum(np.abs(g_o).max(axis=1), 1e-300)
    assert np.all(np.abs(g_g - g_o).max(axis=1) <= GRAD_RTOL * gs)
    hs = np.maximum(np.linalg.norm(H_o, axis=(1, 2)), 1e-300)
    assert np.all(np.linalg.norm(H_g - H_o, axis=(1, 2)) <= HESS_RTOL * hs)
