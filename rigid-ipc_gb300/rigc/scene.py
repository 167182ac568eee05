"""Rigid-body scenes in the reference's JSON scene format, and their set-up.

A scene is a list of rigid bodies.  Each body is built the way the reference
builds one (``src/physics/rigid_body.cpp:43-182``):

* vertices are placed in world space (scale, XYZ Euler rotation in degrees,
  ``src/io/read_rb_scene.cpp:164-200``), then re-centred on the centre of mass
  (``center_vertices``, ``rigid_body.cpp:17-41``);
* mass properties come from the divergence-theorem polyhedral integrals
  (``src/physics/mass.cpp:57-176``, Eberly's published method);
* the rest vertices are expressed in the principal frame ``R0`` of the inertia
  tensor and the pose rotation becomes the rotation vector of ``R0``
  (``rigid_body.cpp:91-131``);
* ``r_max`` is the largest vertex norm and ``average_edge_length`` the mean rest
  edge length (``rigid_body.cpp:164-177``).

Static bodies keep ``R0 = I``: their world geometry is the same either way and
their mass never enters the objective.

Group ids follow ``read_rb_scene.cpp:285-336``: every non-dynamic body shares
one group, every dynamic body without an explicit id gets the next free id.

The flattened arrays (:class:`Scene`) are what the C-ABI's
``rigc_scene_desc`` takes; they mirror ``RigidBodyAssembler::init``
(``src/physics/rigid_body_assembler.cpp:19-118``).
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field

import numpy as np

from . import meshes

BODY_STATIC = 0
BODY_KINEMATIC = 1
BODY_DYNAMIC = 2
_TYPE_NAMES = {"static": BODY_STATIC, "kinematic": BODY_KINEMATIC,
               "dynamic": BODY_DYNAMIC}


# --------------------------------------------------------------------------
# small rotation helpers (scene set-up only; the hot path has its own)

def hat(w):
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


def rotvec_to_matrix(r):
    """R = I + sinc(|r|)[r] + 1/2 sinc^2(|r|/2)[r]^2 (``pose.tpp:203-218``)."""
    r = np.asarray(r, dtype=np.float64)
    th = float(np.linalg.norm(r))
    K = hat(r)
    s = 1.0 if th == 0 else math.sin(th) / th
    s2 = 1.0 if th == 0 else math.sin(th / 2) / (th / 2)
    return np.eye(3) + s * K + 0.5 * s2 * s2 * (K @ K)


def matrix_to_rotvec(R):
    """Angle-axis vector of a rotation matrix (Eigen::AngleAxisd semantics)."""
    c = max(-1.0, min(1.0, (np.trace(R) - 1.0) / 2.0))
    ang = math.acos(c)
    if ang < 1e-12:
        return np.zeros(3)
    if math.pi - ang < 1e-6:
        # near pi: axis from the largest diagonal entry of (R + I) / 2
        B = (R + np.eye(3)) / 2.0
        i = int(np.argmax(np.diag(B)))
        axis = B[:, i] / math.sqrt(B[i, i])
        return axis * ang
    axis = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    axis /= 2.0 * math.sin(ang)
    return axis * ang


def euler_xyz_deg_to_matrix(rot_deg):
    """R = Rz(z) Ry(y) Rx(x), angles in degrees (``read_rb_scene.cpp:189-200``)."""
    x, y, z = np.radians(np.asarray(rot_deg, dtype=np.float64))
    Rx = np.array([[1, 0, 0], [0, math.cos(x), -math.sin(x)], [0, math.sin(x), math.cos(x)]])
    Ry = np.array([[math.cos(y), 0, math.sin(y)], [0, 1, 0], [-math.sin(y), 0, math.cos(y)]])
    Rz = np.array([[math.cos(z), -math.sin(z), 0], [math.sin(z), math.cos(z), 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def matrix_to_euler_xyz_deg(R):
    """Inverse of :func:`euler_xyz_deg_to_matrix`."""
    sy = -R[2, 0]
    sy = max(-1.0, min(1.0, sy))
    y = math.asin(sy)
    if abs(sy) < 1 - 1e-12:
        x = math.atan2(R[2, 1], R[2, 2])
        z = math.atan2(R[1, 0], R[0, 0])
    else:
        x = math.atan2(-R[1, 2], R[1, 1])
        z = 0.0
    return np.degrees([x, y, z])


def random_rotation(rng):
    """Uniform random rotation matrix from a random unit quaternion."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


# --------------------------------------------------------------------------
# mass properties (divergence theorem over a closed triangle mesh)

def mass_properties(V, F):
    """Volume, centre and inertia tensor (about the centre) of a closed mesh."""
    v0, v1, v2 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    N = np.cross(v1 - v0, v2 - v0)

    def sub(w0, w1, w2):
        t0 = w0 + w1
        f1 = t0 + w2
        t1 = w0 * w0
        t2 = t1 + w1 * t0
        f2 = t2 + w2 * f1
        f3 = w0 * t1 + w1 * t2 + w2 * f2
        g0 = f2 + w0 * (f1 + w0)
        g1 = f2 + w1 * (f1 + w1)
        g2 = f2 + w2 * (f1 + w2)
        return f1, f2, f3, g0, g1, g2

    f1x, f2x, f3x, g0x, g1x, g2x = sub(v0[:, 0], v1[:, 0], v2[:, 0])
    f1y, f2y, f3y, g0y, g1y, g2y = sub(v0[:, 1], v1[:, 1], v2[:, 1])
    f1z, f2z, f3z, g0z, g1z, g2z = sub(v0[:, 2], v1[:, 2], v2[:, 2])
    it = np.zeros(10)
    it[0] = np.sum(N[:, 0] * f1x) / 6
    it[1] = np.sum(N[:, 0] * f2x) / 24
    it[2] = np.sum(N[:, 1] * f2y) / 24
    it[3] = np.sum(N[:, 2] * f2z) / 24
    it[4] = np.sum(N[:, 0] * f3x) / 60
    it[5] = np.sum(N[:, 1] * f3y) / 60
    it[6] = np.sum(N[:, 2] * f3z) / 60
    it[7] = np.sum(N[:, 0] * (v0[:, 1] * g0x + v1[:, 1] * g1x + v2[:, 1] * g2x)) / 120
    it[8] = np.sum(N[:, 1] * (v0[:, 2] * g0y + v1[:, 2] * g1y + v2[:, 2] * g2y)) / 120
    it[9] = np.sum(N[:, 2] * (v0[:, 0] * g0z + v1[:, 0] * g1z + v2[:, 0] * g2z)) / 120
    mass = it[0]
    if not (mass > 0 and np.isfinite(mass)):
        raise ValueError("mass properties need a closed, outward-oriented mesh")
    c = it[1:4] / mass
    I = np.array([
        [it[5] + it[6], -it[7], -it[9]],
        [-it[7], it[4] + it[6], -it[8]],
        [-it[9], -it[8], it[4] + it[5]],
    ])
    I[0, 0] -= mass * (c[1] ** 2 + c[2] ** 2)
    I[1, 1] -= mass * (c[2] ** 2 + c[0] ** 2)
    I[2, 2] -= mass * (c[0] ** 2 + c[1] ** 2)
    I[0, 1] += mass * c[0] * c[1]
    I[1, 0] = I[0, 1]
    I[1, 2] += mass * c[1] * c[2]
    I[2, 1] = I[1, 2]
    I[0, 2] += mass * c[2] * c[0]
    I[2, 0] = I[0, 2]
    return mass, c, I


def principal_frame(I):
    """Eigenvalues (ascending) and a rotation whose columns are principal
    axes of the symmetric inertia tensor I (RigidBody's
    SelfAdjointEigenSolver, src/physics/rigid_body.cpp:97-117), made the same
    on every machine: where eigenvalues coincide (within 1e-10 of the
    largest) the axes are not determined by I, so an isotropic tensor takes
    the identity and a two-fold degenerate one the distinct axis completed
    by the world axis least aligned with it; each axis has its largest
    component positive, and the frame is a rotation (det +1)."""
    w, R = np.linalg.eigh(I)
    tol = 1e-10 * max(float(np.abs(w).max()), 1e-300)
    d01, d12 = w[1] - w[0] <= tol, w[2] - w[1] <= tol

    def canon(v):
        v = v / np.linalg.norm(v)
        return v if v[np.argmax(np.abs(v))] > 0 else -v

    if d01 and d12:
        R = np.eye(3)
    elif d01 or d12:
        k = 2 if d01 else 0
        v = canon(R[:, k])
        a = np.eye(3)[int(np.argmin(np.abs(v)))]
        u = canon(a - (a @ v) * v)
        t = np.cross(v, u)
        R = np.column_stack([u, t, v]) if d01 else np.column_stack([v, u, t])
    else:
        R = np.column_stack([canon(R[:, k]) for k in range(3)])
    if np.linalg.det(R) < 0:
        R[:, 0] *= -1.0
    return w, R


# --------------------------------------------------------------------------

@dataclass
class RigidBody:
    name: str
    vertices: np.ndarray          # rest vertices in the body (principal) frame
    edges: np.ndarray
    faces: np.ndarray
    faces_to_edges: np.ndarray
    pose: np.ndarray              # [p(3), theta(3)]
    velocity: np.ndarray          # [v(3) world, omega(3) body frame]
    mass: float
    moment_of_inertia: np.ndarray
    is_dof_fixed: np.ndarray      # 6 bools
    type: int
    group_id: int
    r_max: float = 0.0
    average_edge_length: float = 0.0
    Qdot: np.ndarray = field(default_factory=lambda: np.zeros((3, 3)))
    # kinematic bodies (rigid_body.hpp:260-261): the time the body keeps
    # moving (+inf: always) and the poses (p, theta) it is driven to, one per
    # time step, before its velocity takes over
    kinematic_max_time: float = float("inf")
    kinematic_poses: list = field(default_factory=list)


def make_body(vertices, faces, *, position=(0, 0, 0), rotation_deg=(0, 0, 0),
              scale=1.0, linear_velocity=(0, 0, 0),
              angular_velocity_deg=(0, 0, 0), density=1000.0,
              is_dof_fixed=False, body_type="dynamic", group_id=-1,
              name="RigidBody") -> RigidBody:
    """Build one body from model-space mesh data and JSON-style fields."""
    V = np.asarray(vertices, dtype=np.float64) * np.broadcast_to(
        np.asarray(scale, dtype=np.float64), (3,))
    F = np.asarray(faces, dtype=np.int32)
    R_model = euler_xyz_deg_to_matrix(rotation_deg)
    E = meshes.edges_from_faces(F)
    F2E = meshes.faces_to_edges(F, E)
    if isinstance(is_dof_fixed, (bool, np.bool_)):
        fixed = np.full(6, bool(is_dof_fixed))
    else:
        fixed = np.asarray(is_dof_fixed, dtype=bool).copy()
    btype = _TYPE_NAMES[body_type] if isinstance(body_type, str) else int(body_type)
    if btype == BODY_STATIC:
        fixed[:] = True
    elif fixed.all():
        btype = BODY_STATIC

    pos = np.asarray(position, dtype=np.float64).copy()
    omega = np.radians(np.asarray(angular_velocity_deg, dtype=np.float64))
    vel = np.concatenate([np.asarray(linear_velocity, dtype=np.float64), omega])

    closed = len(F) >= 4 and btype != BODY_STATIC
    if closed:
        # centre on the centre of mass in the model frame, a few passes
        # (center_vertices, src/physics/rigid_body.cpp:16-43)
        V = V + pos
        pos = np.zeros(3)
        for _ in range(10):
            _, com, _ = mass_properties(V, F)
            V = V - com
            pos = pos + com
            if com @ com < 1e-8:
                break
        vol, _, I = mass_properties(V, F)
        mass = vol * density
        thr = np.abs(I).max() * 1e-16
        I = np.where(np.abs(I) > thr, I, 0.0)
        w, R0 = principal_frame(I)
        moment = density * np.abs(w)
        # R = R_pose R0, vertices V R0, omega = R0^T omega0 (rigid_body.cpp:132-141)
        theta = matrix_to_rotvec(R_model @ R0)
        V = V @ R0
        vel[3:] = R0.T @ vel[3:]
    else:
        # open or static mesh: keep the model frame, nominal mass properties
        V = V @ R_model.T
        area = 0.5 * np.linalg.norm(
            np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]), axis=1).sum()
        mass = max(area, 1e-12) * density
        moment = np.full(3, mass)
        theta = np.zeros(3)
    vel[~fixed] = vel[~fixed]
    vel[fixed] = 0.0
    pose = np.concatenate([pos, theta])
    r_max = float(np.linalg.norm(V, axis=1).max())
    ael = float(np.linalg.norm(V[E[:, 0]] - V[E[:, 1]], axis=1).mean()) if len(E) else 0.0
    Q = rotvec_to_matrix(theta)
    return RigidBody(name=name, vertices=V, edges=E, faces=F, faces_to_edges=F2E,
                     pose=pose, velocity=vel, mass=float(mass),
                     moment_of_inertia=moment, is_dof_fixed=fixed, type=btype,
                     group_id=int(group_id), r_max=r_max,
                     average_edge_length=ael, Qdot=Q @ hat(vel[3:]))


def raw_body(vertices, edges=None, faces=None, *, pose=None, body_type="dynamic",
             group_id=-1, name="RigidBody") -> RigidBody:
    """A body whose rest vertices are used as given (no centring, no principal
    frame), with a zero pose unless one is passed -- the bodies of the
    reference's analytic CCD tests (tests/ccd/test_rigid_body_time_of_impact.cpp:
    70-90 cancel the set-up the same way)."""
    V = np.asarray(vertices, dtype=np.float64).reshape(-1, 3)
    F = np.zeros((0, 3), np.int32) if faces is None else np.asarray(faces, np.int32).reshape(-1, 3)
    if edges is None:
        E = meshes.edges_from_faces(F)
    else:
        E = np.asarray(edges, np.int32).reshape(-1, 2)
    F2E = meshes.faces_to_edges(F, E) if len(F) else np.zeros((0, 3), np.int32)
    btype = _TYPE_NAMES[body_type] if isinstance(body_type, str) else int(body_type)
    fixed = np.full(6, btype == BODY_STATIC)
    r_max = float(np.linalg.norm(V, axis=1).max()) if len(V) else 0.0
    ael = float(np.linalg.norm(V[E[:, 0]] - V[E[:, 1]], axis=1).mean()) if len(E) else 0.0
    return RigidBody(name=name, vertices=V, edges=E, faces=F, faces_to_edges=F2E,
                     pose=np.zeros(6) if pose is None else np.asarray(pose, np.float64),
                     velocity=np.zeros(6), mass=1.0, moment_of_inertia=np.ones(3),
                     is_dof_fixed=fixed, type=btype, group_id=int(group_id), r_max=r_max,
                     average_edge_length=ael, Qdot=np.zeros((3, 3)))


def assign_group_ids(bodies):
    """Group ids as ``read_rb_scene.cpp:285-336`` assigns them."""
    static_ids = set()
    for b in bodies:
        if b.type != BODY_DYNAMIC:
            if b.group_id >= 0:
                static_ids.add(b.group_id)
            b.group_id = -1
    taken = sorted(b.group_id for b in bodies if b.group_id >= 0)
    ti, nid, static_gid = 0, 0, -1
    for b in bodies:
        in_static = b.type != BODY_DYNAMIC or b.group_id in static_ids
        if static_gid >= 0 and in_static:
            b.group_id = static_gid
        elif b.group_id < 0:
            while ti < len(taken) and nid >= taken[ti]:
                if nid == taken[ti]:
                    nid += 1
                ti += 1
            b.group_id = nid
            nid += 1
        if static_gid < 0 and in_static:
            static_gid = b.group_id


@dataclass
class Scene:
    """Flattened scene: what ``rigc_ctx_create`` takes, plus solver settings."""
    bodies: list
    timestep: float = 0.01
    dhat: float = 1e-3
    dmin: float = 0.0
    gravity: tuple = (0.0, -9.81, 0.0)
    friction: float = 0.0
    num_steps: int = 100
    name: str = "scene"
    # the CCD trajectory of the line search ("rigid" or "piecewise_linear";
    # CollisionConstraint's own default is rigid)
    trajectory: str = "rigid"

    def __post_init__(self):
        self.refresh()

    def refresh(self):
        nb = len(self.bodies)
        vs, es, fs = [0], [0], [0]
        for b in self.bodies:
            vs.append(vs[-1] + len(b.vertices))
            es.append(es[-1] + len(b.edges))
            fs.append(fs[-1] + len(b.faces))
        self.body_vertex_start = np.array(vs, dtype=np.int32)
        self.body_edge_start = np.array(es, dtype=np.int32)
        self.body_face_start = np.array(fs, dtype=np.int32)
        self.rest_vertices = np.ascontiguousarray(
            np.concatenate([b.vertices for b in self.bodies]) if nb else np.zeros((0, 3)))
        self.edges = np.ascontiguousarray(np.concatenate(
            [b.edges + vs[i] for i, b in enumerate(self.bodies)]).astype(np.int32))
        self.faces = np.ascontiguousarray(np.concatenate(
            [b.faces + vs[i] for i, b in enumerate(self.bodies)]).astype(np.int32))
        self.faces_to_edges = np.ascontiguousarray(np.concatenate(
            [b.faces_to_edges + es[i] for i, b in enumerate(self.bodies)]).astype(np.int32))
        self.group_ids = np.array([b.group_id for b in self.bodies], dtype=np.int32)
        self.body_type = np.array([b.type for b in self.bodies], dtype=np.int32)
        self.r_max = np.array([b.r_max for b in self.bodies], dtype=np.float64)
        ne = len(self.edges)
        self.average_edge_length = float(
            sum(len(b.edges) * b.average_edge_length for b in self.bodies) / max(ne, 1))
        self.mass = np.array([b.mass for b in self.bodies])
        self.moment = np.array([b.moment_of_inertia for b in self.bodies]).reshape(nb, 3)
        self.is_dof_fixed = np.array([b.is_dof_fixed for b in self.bodies]).reshape(nb, 6)
        free = ~self.is_dof_fixed.reshape(-1)
        md = np.concatenate([np.r_[b.mass, b.mass, b.mass, b.moment_of_inertia]
                             for b in self.bodies]) if nb else np.zeros(0)
        self.average_mass = float(md[free].mean()) if free.any() else 1.0

    @property
    def num_bodies(self):
        return len(self.bodies)

    @property
    def num_vertices(self):
        return len(self.rest_vertices)

    def poses(self):
        """Current poses as the flat dof vector x (6 per body, [p, theta])."""
        return np.concatenate([b.pose for b in self.bodies]).astype(np.float64)

    def velocities(self):
        return np.concatenate([b.velocity for b in self.bodies]).astype(np.float64)

    def world_vertices(self, x):
        x = np.asarray(x).reshape(-1, 6)
        out = np.empty_like(self.rest_vertices)
        for i in range(self.num_bodies):
            a, b = self.body_vertex_start[i], self.body_vertex_start[i + 1]
            R = rotvec_to_matrix(x[i, 3:])
            out[a:b] = self.rest_vertices[a:b] @ R.T + x[i, :3]
        return out

    def predictor_poses(self, x0=None, dt=None):
        """Poses after one explicit step of the current velocities.

        The rotation update composes the body-frame angular velocity onto the
        current rotation, so the end pose is a proper rigid motion.
        """
        dt = self.timestep if dt is None else dt
        x0 = self.poses() if x0 is None else np.asarray(x0)
        x0 = x0.reshape(-1, 6)
        x1 = x0.copy()
        for i, b in enumerate(self.bodies):
            if b.type == BODY_STATIC:
                continue
            x1[i, :3] = x0[i, :3] + dt * b.velocity[:3]
            R = rotvec_to_matrix(x0[i, 3:]) @ rotvec_to_matrix(dt * b.velocity[3:])
            x1[i, 3:] = _continuous_rotvec(matrix_to_rotvec(R), x0[i, 3:])
        return x1.reshape(-1)


def _continuous_rotvec(r, ref):
    """Pick the 2*pi-equivalent rotation vector closest to ``ref``."""
    ang = np.linalg.norm(r)
    if ang < 1e-14:
        return r
    axis = r / ang
    best, bestd = r, np.linalg.norm(r - ref)
    for k in (-2, -1, 1, 2):
        c = axis * (ang + 2 * math.pi * k)
        d = np.linalg.norm(c - ref)
        if d < bestd:
            best, bestd = c, d
    return best


# --------------------------------------------------------------------------
# reference-format JSON (subset used by the narrow phase)

def scene_to_json(spec: dict) -> str:
    return json.dumps(spec, indent=1)


def scene_from_json(spec) -> Scene:
    """Build a :class:`Scene` from a reference-format scene (dict or text).

    Bodies may give inline ``vertices``/``faces`` or a ``mesh`` name from the
    generators here (``cube``, ``plane``, ``icosphere``, ``torus``).
    """
    if isinstance(spec, str):
        spec = json.loads(spec)
    rbp = spec.get("rigid_body_problem", spec)
    bodies = []
    for jb in rbp["rigid_bodies"]:
        if not jb.get("enabled", True):
            continue
        mesh = jb.get("mesh", "")
        if mesh:
            V, F = named_mesh(mesh)
        else:
            V = np.asarray(jb["vertices"], dtype=np.float64)
            F = np.asarray(jb["faces"], dtype=np.int32)
        bodies.append(make_body(
            V, F,
            position=jb.get("position", [0, 0, 0]),
            rotation_deg=jb.get("rotation", [0, 0, 0]),
            scale=jb.get("scale", 1.0),
            linear_velocity=jb.get("linear_velocity", [0, 0, 0]),
            angular_velocity_deg=jb.get("angular_velocity", [0, 0, 0]),
            density=jb.get("density", 1000.0),
            is_dof_fixed=jb.get("is_dof_fixed", False),
            body_type=jb.get("type", "dynamic"),
            group_id=jb.get("group_id", -1),
            name=mesh or "RigidBody"))
        # read_rb_scene.cpp:94-101,233-245: a negative max time is +inf; a
        # kinematic pose's position and rotation are taken as given (missing
        # parts zero)
        kmt = float(jb.get("kinematic_max_time", -1))
        bodies[-1].kinematic_max_time = float("inf") if kmt < 0 else kmt
        bodies[-1].kinematic_poses = [
            np.concatenate([np.asarray(q.get("position", [0, 0, 0]), dtype=np.float64),
                            np.asarray(q.get("rotation", [0, 0, 0]), dtype=np.float64)])
            for q in jb.get("kinematic_poses", [])]
    assign_group_ids(bodies)
    dbc = spec.get("distance_barrier_constraint", {})
    return Scene(
        bodies=bodies,
        timestep=spec.get("timestep", 0.01),
        dhat=dbc.get("initial_barrier_activation_distance", 1e-3),
        dmin=dbc.get("minimum_separation_distance", 0.0),
        gravity=tuple(rbp.get("gravity", [0, -9.81, 0])),
        friction=rbp.get("coefficient_friction", 0.0),
        num_steps=int(round(spec.get("max_time", 1.0) / spec.get("timestep", 0.01))),
        name=spec.get("name", "scene"),
        trajectory=dbc.get("trajectory_type", "rigid"))


def named_mesh(name: str):
    base = name.split("/")[-1]
    if base.startswith("cube"):
        return meshes.cube()
    if base.startswith("plane"):
        return meshes.plane(20.0)
    if base.startswith("icosphere"):
        return meshes.icosphere(3, 1.0)
    if base.startswith("torus"):
        return meshes.torus()
    raise ValueError(f"unknown mesh {name!r}")


def _base_spec(dt, dhat, max_steps, mu=0.0):
    return {
        "scene_type": "distance_barrier_rb_problem",
        "solver": "ipc_solver",
        "timestep": dt,
        "max_time": dt * max_steps,
        "distance_barrier_constraint": {
            "detection_method": "hash_grid",
            "trajectory_type": "rigid",
            "initial_barrier_activation_distance": dhat,
            "minimum_separation_distance": 0.0,
            "barrier_type": "ipc",
        },
        "rigid_body_problem": {"gravity": [0, -9.81, 0],
                               "coefficient_friction": mu, "rigid_bodies": []},
    }


def _rb(V, F, **kw):
    d = {"vertices": np.asarray(V).tolist(), "faces": np.asarray(F).tolist()}
    d.update(kw)
    return d


def lattice_rotation(rng, max_deg=2.5):
    """Rotation about a uniformly random axis by an angle U[0, max_deg] degrees.

    Unit cubes whose centres are 1.05 m apart interpenetrate under larger
    rotations (a cube's half-extent along a lattice axis exceeds 0.525 m past
    about 2.9 degrees), so the lattice scenes draw their seeded rotations from
    this range."""
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    return rotvec_to_matrix(axis * math.radians(rng.uniform(0.0, max_deg)))


def spec_cubes(seed=0, n=3, spacing=1.05, vel_sigma=0.5, dt=0.01, dhat=1e-3,
               steps=100):
    """27 (n^3) unit cubes in a lattice above a static 20 x 20 m plane."""
    rng = np.random.default_rng(seed)
    spec = _base_spec(dt, dhat, steps)
    Vc, Fc = meshes.cube()
    bodies = spec["rigid_body_problem"]["rigid_bodies"]
    for i in range(n):
        for j in range(n):
            for k in range(n):
                R = lattice_rotation(rng)
                bodies.append(_rb(
                    Vc, Fc,
                    position=[(i - (n - 1) / 2) * spacing, 1.0 + j * spacing,
                              (k - (n - 1) / 2) * spacing],
                    rotation=matrix_to_euler_xyz_deg(R).tolist(),
                    linear_velocity=rng.normal(0, vel_sigma, 3).tolist()))
    Vp, Fp = meshes.plane(20.0)
    bodies.append(_rb(Vp, Fp, position=[0, 0, 0], is_dof_fixed=True,
                      type="static"))
    return spec


def spec_icospheres(seed=0, n=1000, box=(20.0, 40.0, 20.0), dt=0.01, dhat=1e-3,
                    steps=200, mu=0.5, radii=(0.3, 0.6)):
    """Icospheres (subdivision 3) placed without overlap in a box."""
    rng = np.random.default_rng(seed)
    spec = _base_spec(dt, dhat, steps, mu)
    Vs, Fs = meshes.icosphere(3, 1.0)
    r = rng.uniform(radii[0], radii[1], n)
    centres = []
    cell = 2 * radii[1]
    grid = {}
    for i in range(n):
        for _ in range(10000):
            c = np.array([rng.uniform(-box[0] / 2 + r[i], box[0] / 2 - r[i]),
                          rng.uniform(r[i] + 0.01, box[1] - r[i]),
                          rng.uniform(-box[2] / 2 + r[i], box[2] / 2 - r[i])])
            key = tuple((c // cell).astype(int))
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                            if np.linalg.norm(c - centres[j]) < r[i] + r[j] + 1e-3:
                                ok = False
            if ok:
                break
        centres.append(c)
        grid.setdefault(key, []).append(i)
    bodies = spec["rigid_body_problem"]["rigid_bodies"]
    for i in range(n):
        R = random_rotation(rng)
        bodies.append(_rb(
            Vs * r[i], Fs, position=centres[i].tolist(),
            rotation=matrix_to_euler_xyz_deg(R).tolist(),
            linear_velocity=rng.normal(0, 1.0, 3).tolist(),
            angular_velocity=np.degrees(rng.normal(0, 2.0, 3)).tolist()))
    Vp, Fp = meshes.plane(max(box[0], box[2]))
    bodies.append(_rb(Vp, Fp, position=[0, 0, 0], is_dof_fixed=True, type="static"))
    return spec


def spec_chain(n=200, dt=0.005, dhat=1e-4, steps=400, spacing=1.5):
    """Hanging chain of tori; link 0 fixed, odd links turned 90 deg about x.

    At spacing 1.5 neighbouring links touch: the tubes (major radius 1, minor
    0.25) meet at (0.75 + 1.5 i, 0, 0), where both 48 x 24 meshes have a
    vertex, so the initial distance is zero up to rounding.  A spacing a
    little below 1.5 leaves a gap of (1.5 - spacing) (a larger one makes the
    links interpenetrate)."""
    spec = _base_spec(dt, dhat, steps)
    Vt, Ft = meshes.torus(1.0, 0.25, 48, 24)
    bodies = spec["rigid_body_problem"]["rigid_bodies"]
    for i in range(n):
        d = _rb(Vt, Ft, position=[spacing * i, 0, 0],
                rotation=[90.0 if i % 2 else 0.0, 0, 0])
        if i == 0:
            d["type"] = "kinematic"
            d["is_dof_fixed"] = True
        bodies.append(d)
    return spec


def spec_hulls(seed, n_bodies, dt=0.01, dhat=1e-3, steps=100, points=32):
    """One scene of the batched form: convex hulls dropped onto a plane."""
    rng = np.random.default_rng(seed)
    spec = _base_spec(dt, dhat, steps)
    bodies = spec["rigid_body_problem"]["rigid_bodies"]
    side = int(math.ceil(n_bodies ** (1 / 3)))
    k = 0
    for i in range(side):
        for j in range(side):
            for l in range(side):
                if k >= n_bodies:
                    break
                P = rng.normal(size=(points, 3))
                P /= np.linalg.norm(P, axis=1, keepdims=True)
                V, F = meshes.convex_hull(P)
                s = rng.uniform(0.5, 2.0)
                bodies.append(_rb(
                    V * s, F,
                    position=[(i - side / 2) * 4.5, 2.5 + j * 4.5, (l - side / 2) * 4.5],
                    rotation=matrix_to_euler_xyz_deg(random_rotation(rng)).tolist(),
                    linear_velocity=rng.normal(0, 1.0, 3).tolist()))
                k += 1
    Vp, Fp = meshes.plane(max(20.0, side * 5.0))
    bodies.append(_rb(Vp, Fp, position=[0, 0, 0], is_dof_fixed=True, type="static"))
    return spec


def spec_cube_lattice(seed=0, n=4, spacing=1.05, dt=0.01, dhat=1e-3, steps=50):
    """64 cubes in a 4x4x4 lattice with seeded rotations over a static plane."""
    rng = np.random.default_rng(seed)
    spec = _base_spec(dt, dhat, steps)
    Vc, Fc = meshes.cube()
    bodies = spec["rigid_body_problem"]["rigid_bodies"]
    for i in range(n):
        for j in range(n):
            for k in range(n):
                bodies.append(_rb(
                    Vc, Fc,
                    position=[i * spacing, 1.0 + j * spacing, k * spacing],
                    rotation=matrix_to_euler_xyz_deg(lattice_rotation(rng)).tolist()))
    Vp, Fp = meshes.plane(20.0)
    bodies.append(_rb(Vp, Fp, position=[0, 0, 0], is_dof_fixed=True, type="static"))
    return spec


# --------------------------------------------------------------------------
# synthetic contact-rich narrow-phase states

def spec_slab_stacks(seed=0, nx=8, nz=8, layers=2, size=(1.0, 0.2, 1.0), n=(32, 4, 32),
                     gap=3e-4, pitch=1.2, dt=0.01, dhat=1e-3, steps=100):
    """A contact-heavy scene for the barrier terms: nx x nz columns of
    `layers` tessellated slabs (faces of 32 x 32 quads), each resting `gap`
    above the one below or the floor, every slab shifted by a seeded offset
    in x and z so that the face grids do not line up.  Every vertex of a
    slab's bottom face is within dhat of the face below: the 4 x 4 x 2
    stack has some 1.6 x 10^5 constraints, the 8 x 8 x 2 one 6.4 x 10^5."""
    rng = np.random.default_rng(seed)
    spec = _base_spec(dt, dhat, steps)
    Vs, Fs = meshes.tessellated_box(size, n)
    bodies = spec["rigid_body_problem"]["rigid_bodies"]
    for ix in range(nx):
        for iz in range(nz):
            y = 0.0
            for _ in range(layers):
                off = rng.uniform(-0.02, 0.02, 2)
                y += gap + 0.5 * size[1]
                bodies.append(_rb(Vs, Fs, position=[(ix - (nx - 1) / 2) * pitch + off[0], y,
                                                    (iz - (nz - 1) / 2) * pitch + off[1]]))
                y += 0.5 * size[1]
    Vp, Fp = meshes.plane(max(nx, nz) * pitch + 2.0)
    bodies.append(_rb(Vp, Fp, position=[0, 0, 0], is_dof_fixed=True, type="static"))
    return spec


def packed_pile_poses(scene: Scene, seed=0, gap=2e-4, iters=400):
    """Settle the dynamic bodies of an icosphere scene into a pile on the floor.

    A bounding-sphere relaxation (gravity pull, floor and pairwise
    non-penetration projected with a separation of ``gap``) stands in for the
    state of a settled simulation: many bodies end within a fraction of the
    barrier distance of their neighbours.  Orientations are kept.  Returns
    the new pose vector x.
    """
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    x = scene.poses().reshape(-1, 6).copy()
    dyn = np.array([b.type == BODY_DYNAMIC for b in scene.bodies])
    idx = np.nonzero(dyn)[0]
    r = scene.r_max[idx]
    n = len(idx)
    area = np.pi * np.sum(r ** 2) / 0.6
    L = math.sqrt(area / max(1.0, (n ** (1 / 3))))
    P = np.stack([rng.uniform(-L / 2, L / 2, n),
                  rng.uniform(0, 4 * r.max() * n ** (1 / 3), n) + r,
                  rng.uniform(-L / 2, L / 2, n)], axis=1)
    for it in range(iters):
        P[:, 1] -= 0.02 * r.max()
        P[:, 1] = np.maximum(P[:, 1], r + gap)
        P[:, 0] = np.clip(P[:, 0], -L / 2 + r, L / 2 - r)
        P[:, 2] = np.clip(P[:, 2], -L / 2 + r, L / 2 - r)
        for _ in range(4):
            tree = cKDTree(P)
            pairs = tree.query_pairs(2 * r.max() + gap, output_type="ndarray")
            if len(pairs) == 0:
                break
            a, b = pairs[:, 0], pairs[:, 1]
            d = P[b] - P[a]
            dist = np.linalg.norm(d, axis=1)
            need = r[a] + r[b] + gap * (1.5 if it < iters - 1 else 1.01)
            pen = need - dist
            m = pen > 0
            if not m.any():
                break
            corr = (d[m] / np.maximum(dist[m], 1e-12)[:, None]) * (0.5 * pen[m])[:, None]
            np.add.at(P, a[m], -corr)
            np.add.at(P, b[m], corr)
            P[:, 1] = np.maximum(P[:, 1], r + gap)
    # final strict separation
    for _ in range(200):
        tree = cKDTree(P)
        pairs = tree.query_pairs(2 * r.max() + gap, output_type="ndarray")
        if len(pairs) == 0:
            break
        a, b = pairs[:, 0], pairs[:, 1]
        d = P[b] - P[a]
        dist = np.linalg.norm(d, axis=1)
        pen = (r[a] + r[b] + gap) - dist
        m = pen > 0
        if not m.any():
            break
        corr = (d[m] / np.maximum(dist[m], 1e-12)[:, None]) * (0.5 * pen[m] + 1e-9)[:, None]
        np.add.at(P, a[m], -corr)
        np.add.at(P, b[m], corr)
        P[:, 1] = np.maximum(P[:, 1], r + gap)
    x[idx, :3] = P
    return x.reshape(-1)


def concat_scenes(scenes):
    """Independent scenes as one batched scene: (Scene, scene of each body).
    Bodies keep their group ids (pairs never cross scenes)."""
    bodies, sob = [], []
    for k, sc in enumerate(scenes):
        bodies += list(sc.bodies)
        sob += [k] * len(sc.bodies)
    first = scenes[0]
    return (Scene(bodies=bodies, timestep=first.timestep, dhat=first.dhat, dmin=first.dmin,
                  gravity=first.gravity, name="batched"), np.array(sob, dtype=np.int32))
