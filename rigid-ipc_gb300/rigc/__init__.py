"""rigc: the GB300 (sm_103a) Rigid IPC narrow phase, Python front end.

The compute path is the CUDA library behind the C ABI of ``include/rigc.h``;
this module only moves arrays.  Names follow the reference's interface
(``detect_collision_candidates_rigid``, ``construct_constraint_set``,
``compute_barrier_term``, ``compute_earliest_toi``) so the parity tests read
like the reference's own.  Device memory comes from torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from .scene import BODY_KINEMATIC, Scene  # noqa: F401

__all__ = ["Context", "Scene", "L", "fp64_throughput"]


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("rigc needs a CUDA device")
    return torch


def fp64_throughput(op="dfma", active_lanes=32, iters=4096):
    """FP64 issue throughput of the current device (rigc_fp64_throughput):
    dict with ms, warp-level instructions per second and lane-level GFLOP/s."""
    _torch()
    lib = L.load()
    ms, wi, fl = C.c_double(), C.c_double(), C.c_double()
    L.check(lib.rigc_fp64_throughput({"dfma": 0, "dadd": 1}[op], active_lanes, iters,
                                     C.byref(ms), C.byref(wi), C.byref(fl)),
            "rigc_fp64_throughput")
    return {"op": op, "active_lanes": active_lanes, "ms": ms.value,
            "warp_inst_per_s": wi.value / (ms.value * 1e-3),
            "gflops": fl.value / (ms.value * 1e-3) / 1e9}


class Context:
    """One scene on one GPU (a RigidBodyAssembler plus its device buffers)."""

    def __init__(self, scene: Scene, stream=None, scene_of_body=None):
        """scene_of_body (num_bodies ints, non-decreasing) makes a batched
        context of independent scenes (rigc_ctx_create_batched)."""
        self.lib = L.load()
        self.scene = scene
        torch = _torch()
        self.torch = torch
        self._keep = [
            np.ascontiguousarray(scene.rest_vertices, dtype=np.float64),
            np.ascontiguousarray(scene.edges, dtype=np.int32),
            np.ascontiguousarray(scene.faces, dtype=np.int32),
            np.ascontiguousarray(scene.faces_to_edges, dtype=np.int32),
            np.ascontiguousarray(scene.body_vertex_start, dtype=np.int32),
            np.ascontiguousarray(scene.body_edge_start, dtype=np.int32),
            np.ascontiguousarray(scene.body_face_start, dtype=np.int32),
            np.ascontiguousarray(scene.group_ids, dtype=np.int32),
            np.ascontiguousarray(scene.body_type, dtype=np.int32),
            np.ascontiguousarray(scene.r_max, dtype=np.float64),
        ]
        k = self._keep
        d = L.SceneDesc()
        d.num_bodies = scene.num_bodies
        d.num_vertices = scene.num_vertices
        d.num_edges = len(scene.edges)
        d.num_faces = len(scene.faces)
        d.rest_vertices = k[0].ctypes.data_as(L._d)
        d.edges = k[1].ctypes.data_as(L._i32)
        d.faces = k[2].ctypes.data_as(L._i32)
        d.faces_to_edges = k[3].ctypes.data_as(L._i32)
        d.body_vertex_start = k[4].ctypes.data_as(L._i32)
        d.body_edge_start = k[5].ctypes.data_as(L._i32)
        d.body_face_start = k[6].ctypes.data_as(L._i32)
        d.group_ids = k[7].ctypes.data_as(L._i32)
        d.body_types = k[8].ctypes.data_as(L._i32)
        d.r_max = k[9].ctypes.data_as(L._d)
        d.average_edge_length = scene.average_edge_length
        h = C.c_void_p()
        if scene_of_body is None:
            L.check(self.lib.rigc_ctx_create(C.byref(d), C.byref(h)), "rigc_ctx_create")
            self.num_scenes = 1
        else:
            sob = np.ascontiguousarray(scene_of_body, dtype=np.int32)
            self._keep.append(sob)
            self.scene_of_body = sob
            self.num_scenes = int(sob.max()) + 1 if len(sob) else 1
            L.check(self.lib.rigc_ctx_create_batched(C.byref(d), self.num_scenes, sob.ctypes.data,
                                                     C.byref(h)), "rigc_ctx_create_batched")
        self.h = h
        self._last_counts = (0, 0)
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if getattr(self, "h", None):
            self.lib.rigc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        L.check(self.lib.rigc_set_stream(self.h, C.c_void_p(ptr)), "rigc_set_stream")

    # -- helpers ----------------------------------------------------------
    def device(self, x):
        """float64 CUDA tensor from numpy / tensor."""
        t = self.torch
        if isinstance(x, t.Tensor):
            return x.to(device="cuda", dtype=t.float64).contiguous()
        return t.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device="cuda")

    def copy_out(self, ptr, shape, dtype):
        out = np.empty(shape, dtype=dtype)
        if out.nbytes:
            L.check(self.lib.rigc_copy(self.h, out.ctypes.data, C.c_void_p(ptr), out.nbytes),
                    "rigc_copy")
        return out

    def stats(self):
        s = L.Stats()
        L.check(self.lib.rigc_get_stats(self.h, C.byref(s)), "rigc_get_stats")
        return {f: getattr(s, f) for f, _ in L.Stats._fields_}

    # -- reference-facing operations --------------------------------------
    def world_vertices(self, x):
        xd = self.device(x)
        V = self.torch.empty((self.scene.num_vertices, 3), dtype=self.torch.float64, device="cuda")
        L.check(self.lib.rigc_world_vertices(self.h, C.c_void_p(xd.data_ptr()),
                                             C.c_void_p(V.data_ptr())), "rigc_world_vertices")
        return V

    def detect_collision_candidates_rigid(self, x0, x1=None, continuous=True, inflation=0.0):
        """Hash-grid candidates; returns (ee, fv) as int32 numpy arrays."""
        x0d = self.device(x0)
        x1d = self.device(x0 if x1 is None else x1)
        out = L.Candidates()
        L.check(self.lib.rigc_detect_candidates(self.h, C.c_void_p(x0d.data_ptr()),
                                                C.c_void_p(x1d.data_ptr()), int(continuous),
                                                inflation, C.byref(out)),
                "rigc_detect_candidates")
        self._last_counts = (out.num_ee, out.num_fv)
        ee = self.copy_out(out.ee, (out.num_ee, 2), np.int32)
        fv = self.copy_out(out.fv, (out.num_fv, 2), np.int32)
        return ee, fv

    def count_collision_candidates_rigid(self, x0, x1=None, continuous=True, inflation=0.0):
        """The hash-grid broad phase with the candidates left on the device
        (the next CCD or constraint set takes them); returns (num_ee, num_fv)."""
        x0d = self.device(x0)
        x1d = self.device(x0 if x1 is None else x1)
        out = L.Candidates()
        L.check(self.lib.rigc_detect_candidates(self.h, C.c_void_p(x0d.data_ptr()),
                                                C.c_void_p(x1d.data_ptr()), int(continuous),
                                                inflation, C.byref(out)),
                "rigc_detect_candidates")
        self._last_counts = (out.num_ee, out.num_fv)
        return out.num_ee, out.num_fv

    def scene_tois(self):
        """Per-scene earliest time of impact of the last CCD call."""
        out = np.empty(self.num_scenes)
        L.check(self.lib.rigc_scene_tois(self.h, out.ctypes.data_as(L._d)), "rigc_scene_tois")
        return out

    def scene_barrier_energies(self):
        """Per-scene barrier energy of the last barrier-term call."""
        out = np.empty(self.num_scenes)
        L.check(self.lib.rigc_scene_barrier_energies(self.h, out.ctypes.data_as(L._d)),
                "rigc_scene_barrier_energies")
        return out

    def set_candidates(self, ee, fv):
        """Use the given (edge, edge) and (face, vertex) pairs as the candidate set."""
        ee = np.ascontiguousarray(np.asarray(ee, np.int32).reshape(-1, 2))
        fv = np.ascontiguousarray(np.asarray(fv, np.int32).reshape(-1, 2))
        L.check(self.lib.rigc_set_candidates(self.h, len(ee), ee.ctypes.data if len(ee) else None,
                                             len(fv), fv.ctypes.data if len(fv) else None),
                "rigc_set_candidates")

    def set_ccd_budget(self, max_boxes_per_candidate):
        L.check(self.lib.rigc_set_ccd_budget(self.h, int(max_boxes_per_candidate)),
                "rigc_set_ccd_budget")

    def earliest_toi(self, x0, x1, toi_tol=1e-4, prune=True, per_candidate=False):
        """compute_earliest_toi_narrow_phase over the last continuous candidates."""
        x0d, x1d = self.device(x0), self.device(x1)
        toi = C.c_double()
        per = None
        s = self.stats()
        n = s["cand_ee"] + s["cand_fv"]
        if per_candidate:
            per = self.torch.empty(max(n, 1), dtype=self.torch.float64, device="cuda")
        flags = 0 if prune else L.RIGC_TOI_NO_PRUNE
        st = self.lib.rigc_earliest_toi(self.h, C.c_void_p(x0d.data_ptr()),
                                        C.c_void_p(x1d.data_ptr()), toi_tol, flags,
                                        C.byref(toi),
                                        C.c_void_p(per.data_ptr()) if per is not None else None)
        L.check(st, "rigc_earliest_toi",
                allow=(L.RIGC_ERR_QUEUE_OVERFLOW, L.RIGC_ERR_ITER_LIMIT))
        if per_candidate:
            return toi.value, per[:n].cpu().numpy(), st
        return toi.value

    def compute_earliest_toi(self, x0, x1, dmin=0.0):
        """DistanceBarrierConstraint::compute_earliest_toi (broad + narrow)."""
        x0d, x1d = self.device(x0), self.device(x1)
        toi = C.c_double()
        st = self.lib.rigc_compute_earliest_toi(self.h, C.c_void_p(x0d.data_ptr()),
                                                C.c_void_p(x1d.data_ptr()), dmin, C.byref(toi))
        L.check(st, "rigc_compute_earliest_toi",
                allow=(L.RIGC_ERR_QUEUE_OVERFLOW, L.RIGC_ERR_ITER_LIMIT))
        return toi.value

    def earliest_toi_piecewise_linear(self, x0, x1, dmin=0.0, per_candidate=False):
        """compute_earliest_toi_narrow_phase with trajectory PIECEWISE_LINEAR over
        the last continuous candidates (minimum separation dmin)."""
        x0d, x1d = self.device(x0), self.device(x1)
        toi = C.c_double()
        s = self.stats()
        n = s["cand_ee"] + s["cand_fv"]
        per = self.torch.empty(max(n, 1), dtype=self.torch.float64, device="cuda") if per_candidate else None
        st = self.lib.rigc_earliest_toi_piecewise_linear(
            self.h, C.c_void_p(x0d.data_ptr()), C.c_void_p(x1d.data_ptr()), float(dmin), C.byref(toi),
            C.c_void_p(per.data_ptr()) if per is not None else None)
        L.check(st, "rigc_earliest_toi_piecewise_linear",
                allow=(L.RIGC_ERR_QUEUE_OVERFLOW, L.RIGC_ERR_ITER_LIMIT))
        if per_candidate:
            return toi.value, per[:n].cpu().numpy(), st
        return toi.value

    def set_pl_search(self, per_lane=-1):
        """Piecewise-linear CCD: a candidate per lane (1) or per warp (0, and
        -1: the default)."""
        L.check(self.lib.rigc_set_pl_search(self.h, int(per_lane)), "rigc_set_pl_search")

    def set_ccd_window(self, window_log2=-1):
        """Time windows of the rigid CCD's pruned searches: first window
        2^-window_log2, doubled each launch (-1: the built-in 2^-6 from
        65,536 candidates on, 0: no windows).  The earliest time of impact
        does not depend on it."""
        L.check(self.lib.rigc_set_ccd_window(self.h, int(window_log2)), "rigc_set_ccd_window")

    def compute_earliest_toi_piecewise_linear(self, x0, x1, dmin=0.0):
        """DistanceBarrierConstraint::compute_earliest_toi with trajectory
        PIECEWISE_LINEAR (broad phase with inflation dmin / 2, then the narrow
        phase)."""
        x0d, x1d = self.device(x0), self.device(x1)
        toi = C.c_double()
        st = self.lib.rigc_compute_earliest_toi_piecewise_linear(
            self.h, C.c_void_p(x0d.data_ptr()), C.c_void_p(x1d.data_ptr()), float(dmin), C.byref(toi))
        L.check(st, "rigc_compute_earliest_toi_piecewise_linear",
                allow=(L.RIGC_ERR_QUEUE_OVERFLOW, L.RIGC_ERR_ITER_LIMIT))
        return toi.value

    def construct_constraint_set(self, x, dhat, dmin=0.0):
        """Returns the constraint arrays (numpy): type, verts, prims, bodies, weight, eps."""
        xd = self.device(x)
        v = L.ConstraintsView()
        L.check(self.lib.rigc_construct_constraint_set(self.h, C.c_void_p(xd.data_ptr()), dhat,
                                                       dmin, C.byref(v)),
                "rigc_construct_constraint_set")
        n = v.num
        return dict(
            type=self.copy_out(v.type, (n,), np.int32),
            verts=self.copy_out(v.verts, (n, 4), np.int32),
            prims=self.copy_out(v.prims, (n, 2), np.int32),
            bodies=self.copy_out(v.bodies, (n, 2), np.int32),
            weight=self.copy_out(v.weight, (n,), np.float64),
            eps=self.copy_out(v.eps_x, (n,), np.float64),
            counts=(v.num_vv, v.num_ev, v.num_ee, v.num_fv),
        )

    def compute_min_distance(self, x, dhat, dmin=0.0):
        """DistanceBarrierRBProblem::compute_min_distance(x): the smallest
        constraint distance at x, -1 when the constraint set is empty."""
        xd = self.device(x)
        d = C.c_double()
        L.check(self.lib.rigc_min_distance(self.h, C.c_void_p(xd.data_ptr()), dhat, dmin,
                                           C.byref(d)), "rigc_min_distance")
        return d.value

    def detect_intersections(self, x):
        """RigidBodyProblem::detect_intersections: the number of (edge, face)
        pairs of different bodies that cross at poses x (0: intersection-free)."""
        xd = self.device(x)
        n = C.c_int64()
        L.check(self.lib.rigc_detect_intersections(self.h, C.c_void_p(xd.data_ptr()), C.byref(n)),
                "rigc_detect_intersections")
        return n.value

    def set_constraints(self, types, verts, prims, bodies, weight, eps):
        arrs = [np.ascontiguousarray(types, np.int32), np.ascontiguousarray(verts, np.int32),
                np.ascontiguousarray(prims, np.int32), np.ascontiguousarray(bodies, np.int32),
                np.ascontiguousarray(weight, np.float64), np.ascontiguousarray(eps, np.float64)]
        L.check(self.lib.rigc_set_constraints(self.h, len(arrs[0]),
                                              *[a.ctypes.data for a in arrs]),
                "rigc_set_constraints")

    def compute_barrier_term(self, x, dhat, dmin=0.0, grad=True, hess=True, project=True):
        """Energy, gradient (6 nb) and BSR Hessian (row_ptr, col, val[nnzb, 6, 6])."""
        xd = self.device(x)
        flags = (L.RIGC_GRAD if grad else 0) | (L.RIGC_HESS if hess else 0) | \
                (L.RIGC_PROJECT_PSD if project else 0)
        o = L.BarrierOut()
        L.check(self.lib.rigc_barrier_term(self.h, C.c_void_p(xd.data_ptr()), dhat, dmin, flags,
                                           C.byref(o)), "rigc_barrier_term")
        nb = self.scene.num_bodies
        g = self.copy_out(o.grad, (6 * nb,), np.float64) if grad or hess else None
        H = None
        if hess:
            H = (self.copy_out(o.row_ptr, (nb + 1,), np.int32),
                 self.copy_out(o.col, (o.nnzb,), np.int32),
                 self.copy_out(o.val, (o.nnzb, 6, 6), np.float64))
        return o.energy, g, H

    def barrier_local_terms_device(self, xd, n, dhat, e, g, H, dmin=0.0, project=True):
        """rigc_barrier_local_terms into caller-owned device tensors (energy
        n, gradient n x 12, Hessian n x 144), with device poses; no copy."""
        flags = L.RIGC_GRAD | L.RIGC_HESS | (L.RIGC_PROJECT_PSD if project else 0)
        L.check(self.lib.rigc_barrier_local_terms(self.h, C.c_void_p(xd.data_ptr()), dhat, dmin,
                                                  flags, C.c_void_p(e.data_ptr()),
                                                  C.c_void_p(g.data_ptr()),
                                                  C.c_void_p(H.data_ptr())),
                "rigc_barrier_local_terms")

    def barrier_local_terms(self, x, n, dhat, dmin=0.0, project=True):
        torch = self.torch
        xd = self.device(x)
        e = torch.empty(max(n, 1), dtype=torch.float64, device="cuda")
        g = torch.empty((max(n, 1), 12), dtype=torch.float64, device="cuda")
        H = torch.empty((max(n, 1), 12, 12), dtype=torch.float64, device="cuda")
        flags = L.RIGC_GRAD | L.RIGC_HESS | (L.RIGC_PROJECT_PSD if project else 0)
        L.check(self.lib.rigc_barrier_local_terms(self.h, C.c_void_p(xd.data_ptr()), dhat, dmin,
                                                  flags, C.c_void_p(e.data_ptr()),
                                                  C.c_void_p(g.data_ptr()),
                                                  C.c_void_p(H.data_ptr())),
                "rigc_barrier_local_terms")
        return e[:n].cpu().numpy(), g[:n].cpu().numpy(), H[:n].cpu().numpy()

    # ---- lagged friction (DistanceBarrierRBProblem::update_friction_constraints
    # and compute_friction_term, distance_barrier_rb_problem.cpp:168-188,1469-1572)

    def friction_setup(self, x_t0, dhat, barrier_stiffness, coefficient_friction):
        """Friction constraints from the current constraint set at x_t0; returns their count."""
        xd = self.device(x_t0)
        n = C.c_int64()
        L.check(self.lib.rigc_friction_setup(self.h, C.c_void_p(xd.data_ptr()), dhat,
                                             barrier_stiffness, coefficient_friction,
                                             C.byref(n)), "rigc_friction_setup")
        self._fric_x0 = xd
        return n.value

    def friction_constraints(self):
        """dict: type, verts, bodies, lambda, closest (n x 2), basis (n x 2 x 3), mu."""
        v = L.FrictionView()
        L.check(self.lib.rigc_get_friction(self.h, C.byref(v)), "rigc_get_friction")
        n = v.num
        coef = self.copy_out(v.coef, (n, 9), np.float64) if n else np.zeros((0, 9))
        return {
            "type": self.copy_out(v.type, (n,), np.int32) if n else np.zeros(0, np.int32),
            "verts": self.copy_out(v.verts, (n, 4), np.int32) if n else np.zeros((0, 4), np.int32),
            "bodies": self.copy_out(v.bodies, (n, 2), np.int32) if n else np.zeros((0, 2), np.int32),
            "lambda": coef[:, 0], "closest": coef[:, 1:3], "basis": coef[:, 3:9].reshape(n, 2, 3),
            "mu": v.mu,
        }

    def compute_friction_term(self, x, epsv_times_h, grad=True, hess=True, project=True):
        """Energy, gradient (6 nb) and BSR Hessian (row_ptr, col, val[nnzb, 6, 6])."""
        xd = self.device(x)
        flags = (L.RIGC_GRAD if grad else 0) | (L.RIGC_HESS if hess else 0) | \
                (L.RIGC_PROJECT_PSD if project else 0)
        o = L.BarrierOut()
        L.check(self.lib.rigc_friction_term(self.h, C.c_void_p(xd.data_ptr()), epsv_times_h, flags,
                                            C.byref(o)), "rigc_friction_term")
        nb = self.scene.num_bodies
        g = self.copy_out(o.grad, (6 * nb,), np.float64) if grad or hess else None
        H = None
        if hess:
            H = (self.copy_out(o.row_ptr, (nb + 1,), np.int32),
                 self.copy_out(o.col, (o.nnzb,), np.int32) if o.nnzb else np.zeros(0, np.int32),
                 self.copy_out(o.val, (o.nnzb, 6, 6), np.float64) if o.nnzb else
                 np.zeros((0, 6, 6)))
        return o.energy, g, H

    def friction_local_terms(self, x, n, epsv_times_h, project=True):
        torch = self.torch
        xd = self.device(x)
        e = torch.empty(max(n, 1), dtype=torch.float64, device="cuda")
        g = torch.empty((max(n, 1), 12), dtype=torch.float64, device="cuda")
        H = torch.empty((max(n, 1), 12, 12), dtype=torch.float64, device="cuda")
        flags = L.RIGC_GRAD | L.RIGC_HESS | (L.RIGC_PROJECT_PSD if project else 0)
        L.check(self.lib.rigc_friction_local_terms(self.h, C.c_void_p(xd.data_ptr()), epsv_times_h,
                                                   flags, C.c_void_p(e.data_ptr()),
                                                   C.c_void_p(g.data_ptr()),
                                                   C.c_void_p(H.data_ptr())),
                "rigc_friction_local_terms")
        return e[:n].cpu().numpy(), g[:n].cpu().numpy(), H[:n].cpu().numpy()

    # ---- time stepping (DistanceBarrierRBProblem::simulation_step with the IPC solver)

    def sim_init(self, timestep, gravity, dhat, dmin=0.0, coefficient_friction=0.0,
                 static_friction_speed_bound=1e-3, max_newton_iterations=3000,
                 velocity_conv_tol=1e-2, velocity_conv_tol_abs=False,
                 line_search_lower_bound=1e-12, dhat_epsilon=1e-9,
                 min_barrier_stiffness_scale=1e11, newton_polish=0, ccd_rescale=1.0,
                 poses=None, velocities=None, Qdot=None, world_bbox_diagonal=None,
                 trajectory="rigid"):
        """Start a simulation from the scene's poses, velocities and Qdot (or
        from the given host arrays: poses / velocities nb x 6, Qdot nb x 9).
        world_bbox_diagonal (default: that of the start poses) bounds the
        barrier stiffness; a resumed run passes the one of the scene as read.
        trajectory: the line search's CCD, "rigid" or "piecewise_linear" (the
        reference's JSON default)."""
        sc = self.scene
        V = sc.world_vertices(sc.poses() if poses is None
                              else np.asarray(poses, np.float64).reshape(-1))
        p = L.SimParams()
        p.timestep = timestep
        p.gravity[:] = list(gravity)
        p.dhat, p.dmin = dhat, dmin
        p.coefficient_friction = coefficient_friction
        p.static_friction_speed_bound = static_friction_speed_bound
        p.max_newton_iterations = max_newton_iterations
        p.velocity_conv_tol = velocity_conv_tol
        p.velocity_conv_tol_abs = int(velocity_conv_tol_abs)
        p.line_search_lower_bound = line_search_lower_bound
        p.dhat_epsilon = dhat_epsilon
        p.min_barrier_stiffness_scale = min_barrier_stiffness_scale
        p.average_mass = sc.average_mass
        p.world_bbox_diagonal = (float(np.linalg.norm(V.max(0) - V.min(0)))
                                 if world_bbox_diagonal is None else float(world_bbox_diagonal))
        p.newton_polish = int(newton_polish)
        p.ccd_rescale = float(ccd_rescale)
        p.trajectory_type = {"rigid": 0, "piecewise_linear": 1}[trajectory]
        fixed = np.array([int(sum(1 << k for k in range(6) if b.is_dof_fixed[k]))
                          for b in sc.bodies], dtype=np.int32)
        if Qdot is None:
            Qdot = np.concatenate([b.Qdot.reshape(-1) for b in sc.bodies])
        keep = [np.ascontiguousarray(sc.mass, np.float64),
                np.ascontiguousarray(sc.moment.reshape(-1), np.float64), fixed,
                np.ascontiguousarray(sc.poses() if poses is None else poses,
                                     np.float64).reshape(-1),
                np.ascontiguousarray(sc.velocities() if velocities is None else velocities,
                                     np.float64).reshape(-1),
                np.ascontiguousarray(Qdot, np.float64).reshape(-1)]
        nb = sc.num_bodies
        if keep[3].size != 6 * nb or keep[4].size != 6 * nb or keep[5].size != 9 * nb:
            raise ValueError("sim_init: poses / velocities need nb x 6 values, Qdot nb x 9")
        s = L.SimState(*[k.ctypes.data for k in keep])
        L.check(self.lib.rigc_sim_init(self.h, C.byref(p), C.byref(s)), "rigc_sim_init")
        self.sim_params = p
        # the kinematic bodies' schedules read from the scene
        if self.num_scenes == 1:
            for i, b in enumerate(sc.bodies):
                if b.type == BODY_KINEMATIC and (b.kinematic_poses or np.isfinite(b.kinematic_max_time)):
                    self.sim_set_kinematic(i, b.kinematic_max_time, b.kinematic_poses)
        if self.num_scenes > 1:
            # each scene's average mass (RigidBodyAssembler::average_mass over
            # its free dofs) and initial bounding-box diagonal
            sob = self.scene_of_body
            Vw = sc.world_vertices(keep[3].reshape(nb, 6))
            vs = sc.body_vertex_start
            free = ~sc.is_dof_fixed
            md = np.concatenate([np.c_[sc.mass, sc.mass, sc.mass], sc.moment], 1)
            am = np.ones(self.num_scenes)
            bb = np.ones(self.num_scenes)
            for k in range(self.num_scenes):
                bodies = np.flatnonzero(sob == k)
                f = free[bodies]
                if f.any():
                    am[k] = float(md[bodies][f].mean())
                Vk = Vw[vs[bodies[0]]:vs[bodies[-1] + 1]]
                bb[k] = float(np.linalg.norm(Vk.max(0) - Vk.min(0)))
            self._keep_sim = (am, bb)
            L.check(self.lib.rigc_sim_scene_params(self.h, am.ctypes.data, bb.ctypes.data),
                    "rigc_sim_scene_params")

    def sim_step(self, num_steps=1):
        st = L.StepStats()
        L.check(self.lib.rigc_sim_step(self.h, num_steps, C.byref(st)), "rigc_sim_step")
        return {f: getattr(st, f) for f, _ in L.StepStats._fields_}

    def autotune(self, x0, x1, dhat, dmin=0.0):
        """Choose the narrow phase's launch shapes on this workload (kept for
        later calls); returns the choice and the timings."""
        x0d, x1d = self.device(x0), self.device(x1)
        r = L.TuneReport()
        L.check(self.lib.rigc_autotune(self.h, x0d.data_ptr(), x1d.data_ptr(), dhat, dmin,
                                       C.byref(r)), "rigc_autotune")
        return {f: getattr(r, f) for f, _ in L.TuneReport._fields_}

    def set_tune(self, ccd_blocks_per_sm=0, cache_slots_per_body=0, barrier_per_warp=0,
                 ccd_seeds_log2=-1, ccd_hand_off=-1, ccd_warp=-1):
        L.check(self.lib.rigc_set_tune(self.h, ccd_blocks_per_sm, cache_slots_per_body,
                                       barrier_per_warp, ccd_seeds_log2, ccd_hand_off, ccd_warp),
                "rigc_set_tune")

    def sim_set_kinematic(self, body, max_time=-1.0, poses=()):
        """A kinematic body's schedule: the poses (n x 6) the next steps drive
        it to, then x0 + h v; static once max_time has run out (negative: no
        limit)."""
        q = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 6))
        mt = -1.0 if not np.isfinite(max_time) else float(max_time)
        L.check(self.lib.rigc_sim_set_kinematic(self.h, int(body), mt, len(q),
                                                q.ctypes.data if len(q) else None),
                "rigc_sim_set_kinematic")

    def sim_rollout(self, num_steps, checkpoint_every=10):
        """Advance num_steps steps, keeping checkpoints for sim_backward."""
        st = L.StepStats()
        L.check(self.lib.rigc_sim_rollout(self.h, num_steps, checkpoint_every, C.byref(st)),
                "rigc_sim_rollout")
        return {f: getattr(st, f) for f, _ in L.StepStats._fields_}

    def sim_backward(self, d_poses, d_velocities=None, d_Qdot=None):
        """Gradients with respect to the state before the last rollout from
        those with respect to the state after it: (poses nb x 6, velocities
        nb x 6, Qdot nb x 9)."""
        nb = self.scene.num_bodies
        dp = np.ascontiguousarray(d_poses, np.float64).reshape(nb, 6)
        dv = None if d_velocities is None else np.ascontiguousarray(d_velocities, np.float64).reshape(nb, 6)
        dq = None if d_Qdot is None else np.ascontiguousarray(d_Qdot, np.float64).reshape(nb, 9)
        gp, gv, gq = np.empty((nb, 6)), np.empty((nb, 6)), np.empty((nb, 9))
        L.check(self.lib.rigc_sim_backward(
            self.h, dp.ctypes.data, None if dv is None else dv.ctypes.data,
            None if dq is None else dq.ctypes.data, gp.ctypes.data, gv.ctypes.data,
            gq.ctypes.data), "rigc_sim_backward")
        return gp, gv, gq

    def sim_state(self):
        """(poses[nb, 6], velocities[nb, 6], Qdot[nb, 9], barrier stiffness)."""
        nb = self.scene.num_bodies
        P = np.empty((nb, 6))
        V = np.empty((nb, 6))
        Q = np.empty((nb, 9))
        k = C.c_double()
        L.check(self.lib.rigc_sim_get_state(self.h, P.ctypes.data, V.ctypes.data, Q.ctypes.data,
                                            C.byref(k)), "rigc_sim_get_state")
        return P, V, Q, k.value

    def body_state(self, x_t0=None):
        """Device arrays of the bodies' state at the start of the step."""
        sc = self.scene
        t = self.torch
        dev = dict(device="cuda")
        fixed = np.array([int(sum(1 << k for k in range(6) if b.is_dof_fixed[k]))
                          for b in sc.bodies], dtype=np.int32)
        arrs = dict(
            mass=t.as_tensor(sc.mass, dtype=t.float64, **dev),
            moment=t.as_tensor(sc.moment.reshape(-1), dtype=t.float64, **dev),
            x_t0=self.device(sc.poses() if x_t0 is None else x_t0),
            v_t0=self.device(sc.velocities()),
            Qdot_t0=t.as_tensor(np.concatenate([b.Qdot.reshape(-1) for b in sc.bodies]),
                                dtype=t.float64, **dev),
            dof_fixed=t.as_tensor(fixed, dtype=t.int32, **dev))
        return arrs

    def body_energy(self, x, state=None, h=None):
        """compute_energy_term: (energy, grad[6 nb], hess[nb, 6, 6])."""
        sc = self.scene
        st = self.body_state() if state is None else state
        s = L.BodyState(*[C.c_void_p(st[k].data_ptr()) for k in
                          ("mass", "moment", "x_t0", "v_t0", "Qdot_t0", "dof_fixed")])
        xd = self.device(x)
        t = self.torch
        g = t.empty(6 * sc.num_bodies, dtype=t.float64, device="cuda")
        H = t.empty((sc.num_bodies, 6, 6), dtype=t.float64, device="cuda")
        grav = (C.c_double * 3)(*sc.gravity)
        e = C.c_double()
        L.check(self.lib.rigc_body_energy(self.h, C.byref(s), C.c_void_p(xd.data_ptr()), grav,
                                          sc.timestep if h is None else h, C.byref(e),
                                          C.c_void_p(g.data_ptr()), C.c_void_p(H.data_ptr())),
                "rigc_body_energy")
        return e.value, g.cpu().numpy(), H.cpu().numpy()

    def narrow_phase_host(self, x0, x1, dhat, dmin=0.0, nnzb_cap=None):
        """One host-facing narrow-phase pass (host buffers in and out)."""
        nb = self.scene.num_bodies
        x0 = np.ascontiguousarray(x0, np.float64)
        x1 = np.ascontiguousarray(x1, np.float64)
        cap = nnzb_cap if nnzb_cap is not None else 64 * nb
        grad = np.empty(6 * nb)
        rp = np.empty(nb + 1, np.int32)
        col = np.empty(cap, np.int32)
        val = np.empty((cap, 6, 6))
        toi, energy = C.c_double(), C.c_double()
        nnzb = C.c_int64()
        st = self.lib.rigc_narrow_phase_host(self.h, x0.ctypes.data, x1.ctypes.data, dhat, dmin,
                                             C.byref(toi), C.byref(energy), grad.ctypes.data,
                                             rp.ctypes.data, col.ctypes.data, val.ctypes.data,
                                             cap, C.byref(nnzb))
        L.check(st, "rigc_narrow_phase_host",
                allow=(L.RIGC_ERR_QUEUE_OVERFLOW, L.RIGC_ERR_ITER_LIMIT))
        k = nnzb.value
        return toi.value, energy.value, grad, (rp, col[:k], val[:k]), k
