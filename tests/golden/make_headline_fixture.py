"""Oracle results on the benchmark's headline workload, as a fixture.

The workload is the 1000-icosphere contact pile of bench.make_workload(1000,
0): 1000 subdivision-3 icospheres (radii U[0.3, 0.6]) in a seeded pile with
2e-4 m gaps over a static floor, x0 the pile and x1 one explicit step of the
seeded velocities.  This script runs the CPU oracle on it and stores:

* a digest of the inputs (rest vertices, x0, x1), so a test can tell whether
  its machine built the same scene;
* digests and counts of the continuous candidate set (x0 -> x1, no
  inflation) and the discrete one (x0, inflation dhat / 2);
* the earliest time of impact over every continuous candidate;
* per-candidate times of impact (no cross-candidate pruning) of a seeded
  sample of 20,000 continuous candidates;
  (both with the CUDA path's built-in budget of 2^22 boxes per search);
* the constraint set at x0 (dhat 1e-3), its barrier energy and gradient.

Run from the repository root: python tests/golden/make_headline_fixture.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "rigid-ipc_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

OUT = os.path.join(HERE, "headline_pile_1000.npz")
SAMPLE = 20000
DHAT = 1e-3
# the CUDA path's built-in box budget per candidate search (rigc_set_ccd_budget):
# both sides stop a search that reaches it with the same conservative answer
BUDGET = 1 << 22


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def workload():
    import bench

    return bench.make_workload(1000, 0)


def sample_indices(n_ee, n_fv, k=SAMPLE, seed=7):
    rng = np.random.default_rng(seed)
    sel = np.sort(rng.choice(n_ee + n_fv, size=min(k, n_ee + n_fv), replace=False))
    return sel[sel < n_ee], sel[sel >= n_ee] - n_ee


def oracle_results(sc, x0, x1, nthreads=None):
    import oracle as O

    O.build()
    nthreads = nthreads or os.cpu_count() or 1
    o = O.OracleScene(sc)
    ee, fv = o.detect_candidates(x0, x1, True, 0.0)
    ee_d, fv_d = o.detect_candidates(x0, continuous=False, inflation=DHAT / 2)
    toi = o.earliest_toi(x0, x1, ee, fv, nthreads=nthreads, max_boxes=BUDGET)
    se, sf = sample_indices(len(ee), len(fv))
    _, per, _ = o.earliest_toi(x0, x1, ee[se], fv[sf], per_candidate=True, nthreads=nthreads,
                               max_boxes=BUDGET)
    cs = o.constraint_set(x0, ee_d, fv_d, DHAT)
    energy, grad, _ = o.barrier_term(x0, cs, DHAT)
    return dict(ee=ee, fv=fv, ee_d=ee_d, fv_d=fv_d, toi=toi, sample_ee=se, sample_fv=sf,
                sample_toi=per, cs=cs, energy=energy, grad=grad)


def main():
    sc, x0, x1 = workload()
    r = oracle_results(sc, x0, x1)
    cs = r["cs"]
    np.savez_compressed(
        OUT,
        input_digest=digest(sc.rest_vertices, x0, x1),
        ee_digest=digest(r["ee"]), fv_digest=digest(r["fv"]),
        n_ee=len(r["ee"]), n_fv=len(r["fv"]),
        ee_d_digest=digest(r["ee_d"]), fv_d_digest=digest(r["fv_d"]),
        n_ee_d=len(r["ee_d"]), n_fv_d=len(r["fv_d"]),
        toi=r["toi"], sample_ee=r["sample_ee"], sample_fv=r["sample_fv"],
        sample_toi=r["sample_toi"],
        cs_types=cs.types, cs_verts=cs.verts, cs_prims=cs.prims, cs_bodies=cs.bodies,
        energy=r["energy"], grad=r["grad"])
    print(f"wrote {OUT}: {len(r['ee'])} + {len(r['fv'])} continuous, "
          f"{len(r['ee_d'])} + {len(r['fv_d'])} discrete candidates, toi {r['toi']!r}, "
          f"{len(cs)} constraints")


if __name__ == "__main__":
    main()
