"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference's CPU algorithm for the narrow phase; only
the tests, the smoke check and the CPU-baseline leg of the benchmark use it,
as the checker.  ``build()`` compiles ``oracle/_build/liboracle.so`` with the
committed Makefile.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int)
_c = C.POINTER(C.c_char)
_ll = C.POINTER(C.c_longlong)


def build(force: bool = False) -> str:
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.orc_scene_new.restype = C.c_void_p
        L.orc_scene_new.argtypes = [C.c_int] * 4 + [_d, _i, _i, _i, _i, _i, _i, _i, _i, _d, C.c_double]
        L.orc_scene_free.argtypes = [C.c_void_p]
        L.orc_rotation_matrix.argtypes = [_d, _d]
        L.orc_world_vertices.argtypes = [C.c_void_p, _d, _d]
        L.orc_world_vertices_diff.argtypes = [C.c_void_p, _d, _d, _d, _d]
        L.orc_point_triangle_distance_type.argtypes = [_d] * 4
        L.orc_edge_edge_distance_type.argtypes = [_d] * 4
        L.orc_barrier.restype = C.c_double
        L.orc_barrier.argtypes = [C.c_double, C.c_double]
        L.orc_project_to_psd.argtypes = [C.c_int, _d, _d]
        L.orc_detect_candidates.argtypes = [C.c_void_p, _d, _d, C.c_int, C.c_double, C.c_int,
                                            _i, C.c_longlong, _i, C.c_longlong, _ll, _ll]
        L.orc_close_bodies.restype = C.c_longlong
        L.orc_close_bodies.argtypes = [C.c_void_p, _d, _d, C.c_double, _i, C.c_longlong]
        L.orc_element_aabbs.argtypes = [C.c_void_p, _d, _d, C.c_int, C.c_double, _d, _d, _d,
                                        _c, _c, _c]
        L.orc_constraint_set.argtypes = [C.c_void_p, _d, _i, C.c_longlong, _i, C.c_longlong,
                                         C.c_double, C.c_double, _i, _i, _i, _i, _d, _d,
                                         C.c_longlong, _ll]
        L.orc_detect_intersections.restype = C.c_longlong
        L.orc_detect_intersections.argtypes = [C.c_void_p, _d]
        L.orc_min_distance.restype = C.c_double
        L.orc_min_distance.argtypes = [C.c_void_p, _d, C.c_double, C.c_double]
        L.orc_local_terms.argtypes = [C.c_void_p, _d, C.c_longlong, _i, _i, _i, _i, _d, _d,
                                      C.c_double, C.c_double, C.c_int, _d, _d, _d]
        L.orc_friction_constraints.argtypes = [C.c_void_p, _d, C.c_longlong, _i, _i, _i, _i, _d,
                                               _d, C.c_double, C.c_double, C.c_double, _d, _d, _d]
        L.orc_friction_local_terms.argtypes = [C.c_void_p, _d, _d, C.c_longlong, _i, _i, _i, _i,
                                               _d, _d, _d, _d, _d, C.c_double, C.c_double, C.c_int,
                                               _d, _d, _d]
        L.orc_friction_term.argtypes = [C.c_void_p, _d, _d, C.c_longlong, _i, _i, _i, _i, _d, _d,
                                        _d, _d, _d, C.c_double, C.c_double, C.c_int, _d, _d, _i,
                                        _i, _d, C.c_longlong, _ll]
        L.orc_simulation_step.argtypes = [C.c_void_p, _d, _d, _d, _d, _d, _i, _i, _d, _d, _ll]
        L.orc_simulation_step_rec.argtypes = [C.c_void_p, _d, _d, _d, _d, _d, _i, _i, _d, _d, _ll,
                                              _d, _d, _d]
        L.orc_adjoint_step.argtypes = [C.c_void_p] + [_d] * 5 + [_i, _i] + [_d] * 9
        L.orc_adjoint_step.restype = C.c_int
        L.orc_barrier_term.argtypes = [C.c_void_p, _d, C.c_longlong, _i, _i, _i, _i, _d, _d,
                                       C.c_double, C.c_double, C.c_int, _d, _d, _i, _i, _d,
                                       C.c_longlong, _ll]
        L.orc_body_energy.restype = C.c_double
        L.orc_body_energy.argtypes = [C.c_double, _d, _d, _d, _d, _i, C.c_int, _d, _d,
                                      C.c_double, _d, _d]
        L.orc_edge_edge_toi.argtypes = [C.c_void_p, _d, _d, C.c_int, C.c_int, C.c_double,
                                        C.c_double, _d, _ll]
        L.orc_face_vertex_toi.argtypes = L.orc_edge_edge_toi.argtypes
        L.orc_earliest_toi.restype = C.c_double
        L.orc_earliest_toi.argtypes = [C.c_void_p, _d, _d, _i, C.c_longlong, _i, C.c_longlong,
                                       C.c_double, C.c_int, _d, _ll, C.c_longlong, _i]
        L.orc_pl_toi.argtypes = [C.c_void_p, _d, _d, C.c_int, C.c_int, C.c_int, C.c_double,
                                 C.c_double, _d, _ll]
        L.orc_linear_ccd.argtypes = [C.c_int, _d, _d, C.c_double, _d, _ll]
        L.orc_pl_earliest_toi.restype = C.c_double
        L.orc_pl_earliest_toi.argtypes = [C.c_void_p, _d, _d, _i, C.c_longlong, _i, C.c_longlong,
                                          C.c_double, C.c_int, _d, _ll]
        L.orc_interval_op.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _d]
        L.orc_interval_rotation.argtypes = [_d, _d, _d, _d]
        L.orc_det_sin.restype = C.c_double
        L.orc_det_sin.argtypes = [C.c_double]
        L.orc_det_cos.restype = C.c_double
        L.orc_det_cos.argtypes = [C.c_double]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _dd(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ii(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Constraints:
    """Flat constraint arrays (vv | ev | ee | fv order)."""

    def __init__(self, types, verts, prims, bodies, weight, eps):
        self.types = _ii(types)
        self.verts = _ii(verts).reshape(-1, 4)
        self.prims = _ii(prims).reshape(-1, 2)
        self.bodies = _ii(bodies).reshape(-1, 2)
        self.weight = _dd(weight)
        self.eps = _dd(eps)

    def __len__(self):
        return len(self.types)

    def key_sorted(self):
        """Canonical order: by (type, prim0, prim1)."""
        order = np.lexsort((self.prims[:, 1], self.prims[:, 0], self.types))
        return Constraints(self.types[order], self.verts[order], self.prims[order],
                           self.bodies[order], self.weight[order], self.eps[order])


class OracleScene:
    def __init__(self, scene):
        L = lib()
        self.scene = scene
        self._keep = [
            _dd(scene.rest_vertices), _ii(scene.edges), _ii(scene.faces),
            _ii(scene.faces_to_edges), _ii(scene.body_vertex_start),
            _ii(scene.body_edge_start), _ii(scene.body_face_start),
            _ii(scene.group_ids), _ii(scene.body_type), _dd(scene.r_max)]
        k = self._keep
        self.h = L.orc_scene_new(
            scene.num_bodies, scene.num_vertices, len(scene.edges), len(scene.faces),
            _p(k[0], _d), _p(k[1], _i), _p(k[2], _i), _p(k[3], _i), _p(k[4], _i),
            _p(k[5], _i), _p(k[6], _i), _p(k[7], _i), _p(k[8], _i), _p(k[9], _d),
            scene.average_edge_length)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_scene_free(self.h)
            self.h = None

    def world_vertices(self, x):
        x = _dd(x)
        V = np.empty((self.scene.num_vertices, 3))
        lib().orc_world_vertices(self.h, _p(x, _d), _p(V, _d))
        return V

    def world_vertices_diff(self, x):
        x = _dd(x)
        n = self.scene.num_vertices
        V = np.empty((n, 3))
        dV = np.empty((n, 3, 3))
        d2V = np.empty((n, 3, 3, 3))
        lib().orc_world_vertices_diff(self.h, _p(x, _d), _p(V, _d), _p(dV, _d), _p(d2V, _d))
        return V, dV, d2V

    def detect_candidates(self, x0, x1=None, continuous=True, inflation=0.0, brute=False):
        x0 = _dd(x0)
        x1 = _dd(x0 if x1 is None else x1)
        nee, nfv = C.c_longlong(), C.c_longlong()
        cap = 1 << 16
        while True:
            ee = np.empty((cap, 2), dtype=np.int32)
            fv = np.empty((cap, 2), dtype=np.int32)
            rc = lib().orc_detect_candidates(
                self.h, _p(x0, _d), _p(x1, _d), int(continuous), inflation, int(brute),
                _p(ee, _i), cap, _p(fv, _i), cap, C.byref(nee), C.byref(nfv))
            if rc == 0:
                return ee[:nee.value].copy(), fv[:nfv.value].copy()
            cap = max(nee.value, nfv.value) + 1

    def close_bodies(self, x0, x1, inflation):
        x0, x1 = _dd(x0), _dd(x1)
        cap = self.scene.num_bodies * self.scene.num_bodies
        out = np.empty((max(cap, 1), 2), dtype=np.int32)
        n = lib().orc_close_bodies(self.h, _p(x0, _d), _p(x1, _d), inflation, _p(out, _i), cap)
        return out[:n].copy()

    def element_aabbs(self, x0, x1, continuous, inflation):
        x0, x1 = _dd(x0), _dd(x1)
        s = self.scene
        vb = np.zeros((s.num_vertices, 6))
        eb = np.zeros((len(s.edges), 6))
        fb = np.zeros((len(s.faces), 6))
        vi = np.zeros(s.num_vertices, dtype=np.int8)
        ei = np.zeros(len(s.edges), dtype=np.int8)
        fi = np.zeros(len(s.faces), dtype=np.int8)
        lib().orc_element_aabbs(self.h, _p(x0, _d), _p(x1, _d), int(continuous), inflation,
                                _p(vb, _d), _p(eb, _d), _p(fb, _d), _p(vi, _c), _p(ei, _c),
                                _p(fi, _c))
        return vb, eb, fb, vi.astype(bool), ei.astype(bool), fi.astype(bool)

    def constraint_set(self, x, ee, fv, dhat, dmin=0.0):
        x, ee, fv = _dd(x), _ii(ee), _ii(fv)
        cap = 2 * (len(ee) + len(fv)) + 16
        types = np.empty(cap, np.int32)
        verts = np.empty((cap, 4), np.int32)
        prims = np.empty((cap, 2), np.int32)
        bodies = np.empty((cap, 2), np.int32)
        w = np.empty(cap)
        eps = np.empty(cap)
        n = C.c_longlong()
        rc = lib().orc_constraint_set(
            self.h, _p(x, _d), _p(ee, _i), len(ee), _p(fv, _i), len(fv), dhat, dmin,
            _p(types, _i), _p(verts, _i), _p(prims, _i), _p(bodies, _i), _p(w, _d),
            _p(eps, _d), cap, C.byref(n))
        assert rc == 0
        m = n.value
        return Constraints(types[:m], verts[:m], prims[:m], bodies[:m], w[:m], eps[:m])

    def detect_intersections(self, x):
        """detect_intersections: the number of crossing (edge, face) pairs at x."""
        return int(lib().orc_detect_intersections(self.h, _p(_dd(x), _d)))

    def min_distance(self, x, dhat, dmin=0.0):
        """compute_min_distance(x): the smallest constraint distance at x, -1
        when the constraint set is empty."""
        return lib().orc_min_distance(self.h, _p(_dd(x), _d), dhat, dmin)

    def local_terms(self, x, cs: Constraints, dhat, dmin=0.0, project=True):
        x = _dd(x)
        n = len(cs)
        e = np.empty(n)
        g = np.empty((n, 12))
        H = np.empty((n, 12, 12))
        lib().orc_local_terms(self.h, _p(x, _d), n, _p(cs.types, _i), _p(cs.verts, _i),
                              _p(cs.prims, _i), _p(cs.bodies, _i), _p(cs.weight, _d),
                              _p(cs.eps, _d), dhat, dmin, int(project), _p(e, _d), _p(g, _d),
                              _p(H, _d))
        return e, g, H

    # ---- lagged friction
    def friction_constraints(self, x0, cs: Constraints, dhat, kappa, dmin=0.0):
        """(lambda[n], closest[n, 2], basis[n, 2, 3]) at the start-of-step poses x0."""
        x0 = _dd(x0)
        n = len(cs)
        lam = np.zeros(max(n, 1))
        params = np.zeros((max(n, 1), 2))
        T = np.zeros((max(n, 1), 6))
        lib().orc_friction_constraints(self.h, _p(x0, _d), n, _p(cs.types, _i), _p(cs.verts, _i),
                                       _p(cs.prims, _i), _p(cs.bodies, _i), _p(cs.weight, _d),
                                       _p(cs.eps, _d), dhat, dmin, kappa, _p(lam, _d),
                                       _p(params, _d), _p(T, _d))
        return lam[:n], params[:n], T[:n].reshape(n, 2, 3)

    def _fric_args(self, cs, fc):
        lam, params, T = fc
        n = len(cs)
        lam = _dd(lam) if n else np.zeros(1)
        params = _dd(params).reshape(-1) if n else np.zeros(2)
        T = _dd(T).reshape(-1) if n else np.zeros(6)
        return (n, _p(cs.types, _i), _p(cs.verts, _i), _p(cs.prims, _i), _p(cs.bodies, _i),
                _p(cs.weight, _d), _p(cs.eps, _d), _p(lam, _d), _p(params, _d), _p(T, _d)), \
            (lam, params, T)

    def friction_local_terms(self, x, x0, cs: Constraints, fc, mu, epsvh, project=True):
        x, x0 = _dd(x), _dd(x0)
        n = len(cs)
        e = np.empty(max(n, 1))
        g = np.empty((max(n, 1), 12))
        H = np.empty((max(n, 1), 12, 12))
        args, keep = self._fric_args(cs, fc)
        lib().orc_friction_local_terms(self.h, _p(x, _d), _p(x0, _d), *args, mu, epsvh,
                                       int(project), _p(e, _d), _p(g, _d), _p(H, _d))
        return e[:n], g[:n], H[:n]

    def friction_term(self, x, x0, cs: Constraints, fc, mu, epsvh, project=True):
        x, x0 = _dd(x), _dd(x0)
        nb = self.scene.num_bodies
        grad = np.zeros(6 * nb)
        cap = 4 * len(cs) + 1
        row_ptr = np.zeros(nb + 1, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros((cap, 6, 6))
        energy = C.c_double()
        nnzb = C.c_longlong()
        args, keep = self._fric_args(cs, fc)
        rc = lib().orc_friction_term(self.h, _p(x, _d), _p(x0, _d), *args, mu, epsvh, int(project),
                                     C.byref(energy), _p(grad, _d), _p(row_ptr, _i), _p(col, _i),
                                     _p(val, _d), cap, C.byref(nnzb))
        assert rc == 0
        k = nnzb.value
        return energy.value, grad, (row_ptr, col[:k], val[:k])

    def barrier_term(self, x, cs: Constraints, dhat, dmin=0.0, project=True):
        x = _dd(x)
        nb = self.scene.num_bodies
        grad = np.zeros(6 * nb)
        cap = 4 * len(cs) + 1
        row_ptr = np.zeros(nb + 1, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros((cap, 6, 6))
        energy = C.c_double()
        nnzb = C.c_longlong()
        rc = lib().orc_barrier_term(
            self.h, _p(x, _d), len(cs), _p(cs.types, _i), _p(cs.verts, _i), _p(cs.prims, _i),
            _p(cs.bodies, _i), _p(cs.weight, _d), _p(cs.eps, _d), dhat, dmin, int(project),
            C.byref(energy), _p(grad, _d), _p(row_ptr, _i), _p(col, _i), _p(val, _d), cap,
            C.byref(nnzb))
        assert rc == 0
        k = nnzb.value
        return energy.value, grad, (row_ptr, col[:k].copy(), val[:k].copy())

    def edge_edge_toi(self, x0, x1, ea, eb, bound=1.0, tol=1e-4):
        x0, x1 = _dd(x0), _dd(x1)
        toi, boxes = C.c_double(), C.c_longlong()
        hit = lib().orc_edge_edge_toi(self.h, _p(x0, _d), _p(x1, _d), ea, eb, bound, tol,
                                      C.byref(toi), C.byref(boxes))
        return bool(hit), toi.value, boxes.value

    def face_vertex_toi(self, x0, x1, f, v, bound=1.0, tol=1e-4):
        x0, x1 = _dd(x0), _dd(x1)
        toi, boxes = C.c_double(), C.c_longlong()
        hit = lib().orc_face_vertex_toi(self.h, _p(x0, _d), _p(x1, _d), f, v, bound, tol,
                                        C.byref(toi), C.byref(boxes))
        return bool(hit), toi.value, boxes.value

    def pl_toi(self, x0, x1, kind, a, b, bound=1.0, dmin=0.0):
        """Piecewise-linear time of impact of one candidate (kind 0: edges a,
        b; kind 1: face a, vertex b): (hit, toi, {boxes, pieces, status})."""
        x0, x1 = _dd(x0), _dd(x1)
        toi = C.c_double()
        st = np.zeros(3, np.int64)
        hit = lib().orc_pl_toi(self.h, _p(x0, _d), _p(x1, _d), int(kind), int(a), int(b),
                               float(bound), float(dmin), C.byref(toi), _p(st, _ll))
        return bool(hit), toi.value, dict(boxes=int(st[0]), pieces=int(st[1]), status=int(st[2]))

    def pl_earliest_toi(self, x0, x1, ee, fv, dmin=0.0, nthreads=1):
        """Piecewise-linear earliest time of impact over the candidates:
        (toi, per-candidate tois (ee first), {boxes, pieces, status})."""
        x0, x1, ee, fv = _dd(x0), _dd(x1), _ii(ee), _ii(fv)
        per = np.empty(len(ee) + len(fv))
        st = np.zeros(3, np.int64)
        t = lib().orc_pl_earliest_toi(self.h, _p(x0, _d), _p(x1, _d), _p(ee, _i), len(ee),
                                      _p(fv, _i), len(fv), float(dmin), int(nthreads),
                                      _p(per, _d), _p(st, _ll))
        return t, per, dict(boxes=int(st[0]), pieces=int(st[1]), status=int(st[2]))

    def earliest_toi(self, x0, x1, ee, fv, tol=1e-4, nthreads=1, per_candidate=False,
                     max_boxes=0, with_status=False):
        """Earliest time of impact (per candidate too with per_candidate=True).
        max_boxes > 0 caps each candidate's search as the CUDA path does;
        with_status=True appends the worst status (5 = budget exhausted)."""
        x0, x1, ee, fv = _dd(x0), _dd(x1), _ii(ee), _ii(fv)
        per = np.empty(len(ee) + len(fv)) if per_candidate else None
        boxes = C.c_longlong()
        status = C.c_int()
        t = lib().orc_earliest_toi(self.h, _p(x0, _d), _p(x1, _d), _p(ee, _i), len(ee),
                                   _p(fv, _i), len(fv), tol, nthreads,
                                   _p(per, _d) if per is not None else None, C.byref(boxes),
                                   int(max_boxes), C.byref(status))
        out = (t, per, boxes.value) if per_candidate else (t,)
        if with_status:
            out = out + (status.value,)
        return out if len(out) > 1 else out[0]


def rotation_matrix(theta):
    th = _dd(theta)
    R = np.empty(9)
    lib().orc_rotation_matrix(_p(th, _d), _p(R, _d))
    return R.reshape(3, 3)


def project_to_psd(A):
    A = _dd(A)
    n = A.shape[0]
    out = np.empty_like(A)
    lib().orc_project_to_psd(n, _p(A, _d), _p(out, _d))
    return out


def barrier(d, s):
    return lib().orc_barrier(d, s)


def point_triangle_distance_type(p, t0, t1, t2):
    return lib().orc_point_triangle_distance_type(*[_p(_dd(a), _d) for a in (p, t0, t1, t2)])


def edge_edge_distance_type(a0, a1, b0, b1):
    return lib().orc_edge_edge_distance_type(*[_p(_dd(a), _d) for a in (a0, a1, b0, b1)])


_OPS = {"add": 0, "sub": 1, "mul": 2, "div": 3, "sqrt": 4, "cos": 5, "sin": 6,
        "sinc": 7, "abs": 8}


def interval_op(op, a, b=(0.0, 0.0)):
    out = np.empty(2)
    lib().orc_interval_op(_OPS[op], float(a[0]), float(a[1]), float(b[0]), float(b[1]),
                          _p(out, _d))
    return out[0], out[1]


def interval_rotation(rlo, rhi):
    rlo, rhi = _dd(rlo), _dd(rhi)
    lo, hi = np.empty(9), np.empty(9)
    lib().orc_interval_rotation(_p(rlo, _d), _p(rhi, _d), _p(lo, _d), _p(hi, _d))
    return lo.reshape(3, 3), hi.reshape(3, 3)


def det_sin(x):
    return lib().orc_det_sin(float(x))


def det_cos(x):
    return lib().orc_det_cos(float(x))


SIM_DEFAULTS = dict(dmin=0.0, mu=0.0, epsv=1e-3, max_newton_iterations=3000,
                    velocity_conv_tol=1e-2, velocity_conv_tol_abs=0,
                    line_search_lower_bound=1e-12, dhat_epsilon=1e-9,
                    min_barrier_stiffness_scale=1e11, newton_polish=0, ccd_rescale=1.0,
                    trajectory=0)


def linear_ccd(p0, p1, ms=0.0, fv=False):
    """The piecewise-linear CCD's linear CCD alone: the four points p0 -> p1
    (EE a0 a1 b0 b1; FV v f0 f1 f2) on straight lines over t in [0, 1]:
    (hit, toi, boxes, status)."""
    p0, p1 = _dd(np.asarray(p0, np.float64).reshape(12)), _dd(np.asarray(p1, np.float64).reshape(12))
    toi = C.c_double()
    st = np.zeros(3, np.int64)
    hit = lib().orc_linear_ccd(1 if fv else 0, _p(p0, _d), _p(p1, _d), float(ms), C.byref(toi),
                               _p(st, _ll))
    return bool(hit), toi.value, int(st[0]), int(st[2])


class OracleSim:
    """Time stepping of a scene with the oracle's restated IPC Newton solver.
    State: poses (nb x 6), linear/angular velocities (nb x 6), Qdot (nb x 9),
    barrier stiffness (1 before the first step, as the reference starts)."""

    def __init__(self, scene, h, gravity, dhat, **kw):
        self.scene = scene
        self.o = OracleScene(scene)
        self.p = dict(SIM_DEFAULTS)
        self.p.update(kw)
        self.h, self.gravity, self.dhat = h, _dd(gravity), dhat
        sc = scene
        self.mass = _dd(sc.mass)
        self.moment = _dd(sc.moment.reshape(-1))
        self.fixed = _ii(np.asarray(sc.is_dof_fixed, np.int32).reshape(-1))
        self.type = _ii(sc.body_type)
        self.pose = _dd(sc.poses()).copy()
        self.vel = _dd(sc.velocities()).copy()
        self.Qdot = _dd(np.concatenate([b.Qdot.reshape(-1) for b in sc.bodies])).copy()
        V = sc.world_vertices(self.pose)
        self.bbox_diagonal = float(np.linalg.norm(V.max(0) - V.min(0)))
        self.kappa = C.c_double(1.0)
        self.stats = np.zeros(4, np.int64)
        self.tape = []
        # kinematic schedules (rigid_body.hpp:260-261): the time a kinematic
        # body keeps moving (+inf: always) and the poses it is driven to, one
        # per step
        nb = len(self.mass)
        self.kin_max_time = np.full(nb, np.inf)
        self.kin_poses = [[] for _ in range(nb)]
        for b, body in enumerate(sc.bodies):
            if self.type[b] == 1:
                self.set_kinematic(b, getattr(body, "kinematic_max_time", np.inf),
                                   getattr(body, "kinematic_poses", ()))

    def set_kinematic(self, body, max_time=np.inf, poses=()):
        """A kinematic body's schedule: it becomes static once max_time has
        run out (a negative max_time reads as +inf, as read_rb_scene does), and
        each step drives it to the next pose of the list (x0 + h v once the
        list is empty)."""
        assert self.type[body] == 1, "only kinematic bodies have a schedule"
        self.kin_max_time[body] = np.inf if max_time < 0 else float(max_time)
        self.kin_poses[body] = [np.asarray(q, np.float64).reshape(6).copy() for q in poses]

    def _kinematic_targets(self):
        """init_augmented_lagrangian (distance_barrier_rb_problem.cpp:190-234):
        kinematic bodies whose time has run out become static
        (RigidBody::convert_to_static, rigid_body.hpp:186-193: every dof
        fixed, velocity zero); the others' targets, NaN for none."""
        nb = len(self.mass)
        tgt = np.full(6 * nb, np.nan)
        for b in range(nb):
            if self.type[b] != 1:
                continue
            if self.kin_max_time[b] < 0:
                self.type[b] = 0
                self.fixed[6 * b:6 * b + 6] = 1
                self.vel[6 * b:6 * b + 6] = 0.0
            elif self.kin_poses[b]:
                tgt[6 * b:6 * b + 6] = self.kin_poses[b][0]
        return tgt

    def _advance_kinematic(self):
        """step_kinematic_bodies (distance_barrier_rb_problem.cpp:237-251)."""
        for b in range(len(self.mass)):
            if self.type[b] != 1:
                continue
            if self.kin_max_time[b] < 0:
                self.type[b] = 0
                self.fixed[6 * b:6 * b + 6] = 1
                self.vel[6 * b:6 * b + 6] = 0.0
            else:
                self.kin_max_time[b] -= self.h
                if self.kin_poses[b]:
                    self.kin_poses[b].pop(0)

    def params(self):
        p = self.p
        return _dd([self.h, *self.gravity, self.dhat, p["dmin"], p["mu"], p["epsv"],
                    p["max_newton_iterations"], p["velocity_conv_tol"],
                    p["velocity_conv_tol_abs"], p["line_search_lower_bound"],
                    p["dhat_epsilon"], p["min_barrier_stiffness_scale"], self.bbox_diagonal,
                    self.scene.average_mass, p["newton_polish"], p["ccd_rescale"],
                    p["trajectory"]])

    def step(self, record=False):
        """One time step; with record=True the start-of-step state and the
        step's solution are kept for backward()."""
        prm = self.params()
        st = np.zeros(4, np.int64)
        if record:
            pre = (self.pose.copy(), self.vel.copy(), self.Qdot.copy())
            x = np.empty(len(self.pose))
            rec = np.empty(2)
        else:
            x = rec = None
        tgt = self._kinematic_targets()
        lib().orc_simulation_step_rec(self.o.h, _p(self.mass, _d), _p(self.moment, _d),
                                      _p(self.pose, _d), _p(self.vel, _d), _p(self.Qdot, _d),
                                      _p(self.fixed, _i), _p(self.type, _i), _p(prm, _d),
                                      C.byref(self.kappa), st.ctypes.data_as(_ll),
                                      None if x is None else _p(x, _d),
                                      None if rec is None else _p(rec, _d), _p(tgt, _d))
        self._advance_kinematic()
        if record:
            self.tape.append((pre, x, rec))
        self.stats += st
        return st

    def rollout(self, steps, record=True):
        self.tape = []
        for _ in range(steps):
            self.step(record=record)

    def backward(self, d_pose, d_vel=None, d_Qdot=None):
        """Gradients of a loss with respect to the state before the recorded
        steps, from its gradients with respect to the state after them
        (poses nb x 6, velocities nb x 6, Qdot nb x 9)."""
        nb = len(self.mass)
        dp = _dd(np.asarray(d_pose, np.float64).reshape(-1)).copy()
        dv = np.zeros(6 * nb) if d_vel is None else _dd(np.asarray(d_vel).reshape(-1)).copy()
        dq = np.zeros(9 * nb) if d_Qdot is None else _dd(np.asarray(d_Qdot).reshape(-1)).copy()
        prm = self.params()
        for (pose, vel, Qdot), x, rec in reversed(self.tape):
            op, ov, oq = np.empty_like(dp), np.empty_like(dv), np.empty_like(dq)
            rc = lib().orc_adjoint_step(self.o.h, _p(self.mass, _d), _p(self.moment, _d),
                                        _p(pose, _d), _p(vel, _d), _p(Qdot, _d),
                                        _p(self.fixed, _i), _p(self.type, _i), _p(prm, _d),
                                        _p(x, _d), _p(rec, _d), _p(dp, _d), _p(dv, _d), _p(dq, _d),
                                        _p(op, _d), _p(ov, _d), _p(oq, _d))
            if rc != 0:
                raise RuntimeError("adjoint: singular Hessian of the free dofs, or kinematic bodies")
            dp, dv, dq = op, ov, oq
        return dp.reshape(nb, 6), dv.reshape(nb, 6), dq.reshape(nb, 9)


def body_energy(body, x6, gravity, h):
    g = np.empty(6)
    H = np.empty((6, 6))
    mom = _dd(body.moment_of_inertia)
    pose = _dd(body.pose)
    vel = _dd(body.velocity)
    Qd = _dd(body.Qdot.reshape(-1))
    fixed = _ii(body.is_dof_fixed.astype(np.int32))
    x6 = _dd(x6)
    grav = _dd(gravity)
    e = lib().orc_body_energy(body.mass, _p(mom, _d), _p(pose, _d), _p(vel, _d), _p(Qd, _d),
                              _p(fixed, _i), int(body.type), _p(x6, _d), _p(grav, _d), h,
                              _p(g, _d), _p(H, _d))
    return e, g, H
