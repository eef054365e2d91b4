"""Seeded synthetic scenes for the PlayRho world-step workloads.

A scene is plain columnar data (numpy float32/int32), so the same bytes feed the
CUDA world step, the CPU oracle and the reference driver.  Polygon vertices are
stored in the order the reference's ``PolygonShapeConf::Set`` leaves them:
de-duplicated by ``VertexSet`` (minimum separation = linear slop) and ordered by
the gift-wrapping hull of ``GetConvexHullAsVector`` (DistanceProxy.cpp:62-105),
starting at the lowest right-most vertex and going counter-clockwise.  That
order fixes the contact-feature indices, which parity compares exactly.

No public dataset is involved; generators follow the five workload
descriptions (pyramid, 100k-shape box, 4096 batched worlds, differentiable push,
chains with revolute joints) with fixed seeds.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List

import numpy as np

F32 = np.float32

STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
DISK, POLYGON, EDGE = 0, 1, 2
# Joint kinds (the reference's JointConf types) and their parameters in joint_extra.
JOINT_REVOLUTE, JOINT_DISTANCE, JOINT_ROPE, JOINT_WELD, JOINT_FRICTION, JOINT_MOTOR = 0, 1, 2, 3, 4, 5
JOINT_PRISMATIC, JOINT_WHEEL, JOINT_PULLEY, JOINT_TARGET, JOINT_GEAR = 6, 7, 8, 9, 10
JOINT_PARAMS = {
    JOINT_DISTANCE: ("length", "frequency", "damping_ratio"),
    JOINT_ROPE: ("max_length",),
    JOINT_WELD: ("reference_angle", "frequency", "damping_ratio"),
    JOINT_FRICTION: ("max_force", "max_torque"),
    JOINT_MOTOR: ("linear_offset_x", "linear_offset_y", "angular_offset", "max_force", "max_torque",
                  "correction_factor"),
    JOINT_PRISMATIC: ("axis_x", "axis_y", "reference_angle", "lower", "upper", "motor_speed", "max_motor_force"),
    JOINT_WHEEL: ("axis_x", "axis_y", "motor_speed", "max_motor_torque", "frequency", "damping_ratio"),
    JOINT_PULLEY: ("ground_a_x", "ground_a_y", "ground_b_x", "ground_b_y", "length_a", "length_b", "ratio"),
    JOINT_TARGET: ("target_x", "target_y", "max_force", "frequency", "damping_ratio"),
    # the gear's parameters are the two joints it couples (joint indices of the
    # same scene) and the ratio: GetGearJointConf(world, joint1, joint2, ratio)
    JOINT_GEAR: ("joint1", "joint2", "ratio"),
}
# Parameter defaults of the reference's JointConf types where they are not zero.
JOINT_DEFAULTS = {
    JOINT_MOTOR: {"correction_factor": 0.2},                               # MotorJointConf.hpp
    JOINT_PRISMATIC: {"axis_x": 1.0},                                      # UnitVec::GetRight()
    JOINT_WHEEL: {"axis_x": 1.0, "frequency": 2.0, "damping_ratio": 0.7},  # WheelJointConf.hpp:76-79
    JOINT_PULLEY: {"ratio": 1.0},                                          # PulleyJointConf.hpp:126
    JOINT_TARGET: {"frequency": 5.0, "damping_ratio": 0.7},                # TargetJointConf.hpp:63-69
}
# Body flags (BodyConf booleans): allowSleep, awake, fixedRotation, enabled, bullet.
BF_ALLOW_SLEEP, BF_AWAKE, BF_FIXED_ROTATION, BF_ENABLED, BF_BULLET = 1, 2, 4, 8, 16
BF_DEFAULT = BF_ALLOW_SLEEP | BF_AWAKE | BF_ENABLED

DEFAULT_LINEAR_SLOP = F32(0.005)
DEFAULT_VERTEX_RADIUS = F32(DEFAULT_LINEAR_SLOP * F32(2))  # PolygonShapeConf.hpp:68


@dataclasses.dataclass
class Scene:
    """One world: bodies, shapes (one child each) and joints."""

    body_type: np.ndarray      # int32 [B]
    body_pos: np.ndarray       # float32 [B,3] x, y, angle
    body_vel: np.ndarray       # float32 [B,3] vx, vy, w
    body_acc: np.ndarray       # float32 [B,3] ax, ay, alpha
    body_damp: np.ndarray      # float32 [B,2] linear, angular
    body_flags: np.ndarray     # uint32 [B]
    shape_body: np.ndarray     # int32 [S]
    shape_kind: np.ndarray     # int32 [S]
    shape_voff: np.ndarray     # int32 [S]
    shape_nv: np.ndarray       # int32 [S]
    shape_radius: np.ndarray   # float32 [S]
    shape_density: np.ndarray  # float32 [S]
    shape_friction: np.ndarray  # float32 [S]
    shape_restitution: np.ndarray  # float32 [S]
    shape_filter: np.ndarray   # int32 [S,4] category, mask, group, sensor
    verts: np.ndarray          # float32 [V,2]
    joint_bodies: np.ndarray   # int32 [J,2]
    joint_anchors: np.ndarray  # float32 [J,4] localAnchorA.xy localAnchorB.xy
    joint_params: np.ndarray   # float32 [J,6] refAngle lower upper motorSpeed maxMotorTorque pad
    joint_flags: np.ndarray    # int32 [J,3] enableLimit enableMotor collideConnected
    # joint kind (JOINT_*) and the other kinds' parameters (layouts at JOINT_PARAMS)
    joint_type: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    joint_extra: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 8), np.float32))
    # multi-child shapes (ChainShapeConf, MultiShapeConf): each child is a shape here,
    # with the index of its shape's first child; -1 for a shape of one child
    shape_owner: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))

    def __post_init__(self):
        nj = int(np.asarray(self.joint_bodies).reshape(-1, 2).shape[0])
        if len(self.joint_type) != nj:
            self.joint_type = np.zeros(nj, np.int32)
        if len(self.joint_extra) != nj:
            self.joint_extra = np.zeros((nj, 8), np.float32)
        ns = int(np.asarray(self.shape_body).shape[0])
        if len(self.shape_owner) != ns:
            self.shape_owner = np.full(ns, -1, np.int32)

    @property
    def n_bodies(self) -> int:
        return int(self.body_type.shape[0])

    @property
    def n_shapes(self) -> int:
        return int(self.shape_body.shape[0])

    @property
    def n_joints(self) -> int:
        return int(self.joint_bodies.shape[0])

    def n_dynamic(self) -> int:
        return int(np.count_nonzero(self.body_type == DYNAMIC))


class SceneBuilder:
    """Accumulates bodies/shapes/joints in creation order (= reference IDs)."""

    def __init__(self) -> None:
        self.b_type: List[int] = []
        self.b_pos: List[tuple] = []
        self.b_vel: List[tuple] = []
        self.b_acc: List[tuple] = []
        self.b_damp: List[tuple] = []
        self.b_flags: List[int] = []
        self.s_body: List[int] = []
        self.s_kind: List[int] = []
        self.s_voff: List[int] = []
        self.s_nv: List[int] = []
        self.s_radius: List[float] = []
        self.s_density: List[float] = []
        self.s_friction: List[float] = []
        self.s_rest: List[float] = []
        self.s_filter: List[tuple] = []
        self.verts: List[tuple] = []
        self.j_bodies: List[tuple] = []
        self.j_anchor: List[tuple] = []
        self.j_params: List[tuple] = []
        self.j_flags: List[tuple] = []
        self.j_type: List[int] = []
        self.j_extra: List[tuple] = []
        self.s_owner: List[int] = []

    @classmethod
    def from_scene(cls, sc: "Scene") -> "SceneBuilder":
        """A builder holding ``sc``'s bodies, shapes and joints (same IDs), to add to."""
        sb = cls()
        for b in range(sc.n_bodies):
            sb.body(int(sc.body_type[b]), *(float(v) for v in sc.body_pos[b]), v=tuple(float(v) for v in sc.body_vel[b]),
                    acc=tuple(float(v) for v in sc.body_acc[b]), damp=tuple(float(v) for v in sc.body_damp[b]),
                    flags=int(sc.body_flags[b]))
        for k in range(sc.n_shapes):
            o, n = int(sc.shape_voff[k]), int(sc.shape_nv[k])
            sb._shape(int(sc.shape_body[k]), int(sc.shape_kind[k]), [tuple(v) for v in sc.verts[o:o + n]],
                      float(sc.shape_radius[k]), float(sc.shape_density[k]), float(sc.shape_friction[k]),
                      float(sc.shape_restitution[k]), tuple(int(v) for v in sc.shape_filter[k]))
            sb.s_owner[k] = int(sc.shape_owner[k])
        for j in range(sc.n_joints):
            sb.j_bodies.append(tuple(int(v) for v in sc.joint_bodies[j]))
            sb.j_anchor.append(tuple(float(v) for v in sc.joint_anchors[j]))
            sb.j_params.append(tuple(float(v) for v in sc.joint_params[j]))
            sb.j_flags.append(tuple(int(v) for v in sc.joint_flags[j]))
            sb.j_type.append(int(sc.joint_type[j]))
            sb.j_extra.append(tuple(float(v) for v in sc.joint_extra[j]))
        return sb

    def body(self, btype, x, y, angle=0.0, v=(0.0, 0.0, 0.0), acc=(0.0, 0.0, 0.0),
             damp=(0.0, 0.0), flags=BF_DEFAULT) -> int:
        self.b_type.append(int(btype))
        self.b_pos.append((x, y, angle))
        self.b_vel.append(tuple(v))
        self.b_acc.append(tuple(acc))
        self.b_damp.append(tuple(damp))
        self.b_flags.append(int(flags))
        return len(self.b_type) - 1

    def _shape(self, body, kind, verts, radius, density, friction, restitution, filt):
        self.s_body.append(int(body))
        self.s_kind.append(int(kind))
        self.s_voff.append(len(self.verts))
        self.s_nv.append(len(verts))
        self.verts.extend((float(F32(a)), float(F32(b))) for a, b in verts)
        self.s_radius.append(radius)
        self.s_density.append(density)
        self.s_friction.append(friction)
        self.s_rest.append(restitution)
        self.s_filter.append(filt)
        self.s_owner.append(-1)
        return len(self.s_body) - 1

    def disk(self, body, radius, loc=(0.0, 0.0), density=0.0, friction=0.2, restitution=0.0,
             filt=(1, 0xFFFF, 0, 0)):
        return self._shape(body, DISK, [loc], radius, density, friction, restitution, filt)

    def polygon(self, body, points, vertex_radius=float(DEFAULT_VERTEX_RADIUS), density=0.0,
                friction=0.2, restitution=0.0, filt=(1, 0xFFFF, 0, 0)):
        return self._shape(body, POLYGON, convex_hull(points), vertex_radius, density, friction,
                           restitution, filt)

    def box(self, body, hx, hy, **kw):
        # PolygonShapeConf::SetAsBox vertex order (PolygonShapeConf.cpp:45-55), which is
        # also the hull order.
        return self.polygon(body, [(hx, -hy), (hx, hy), (-hx, hy), (-hx, -hy)], **kw)

    def edge(self, body, v0, v1, vertex_radius=float(DEFAULT_VERTEX_RADIUS), density=0.0,
             friction=0.2, restitution=0.0, filt=(1, 0xFFFF, 0, 0)):
        return self._shape(body, EDGE, [v0, v1], vertex_radius, density, friction, restitution, filt)

    def chain(self, body, points, vertex_radius=float(DEFAULT_VERTEX_RADIUS), density=0.0, friction=0.2,
              restitution=0.0, filt=(1, 0xFFFF, 0, 0)) -> int:
        """ChainShapeConf over `points` (a loop repeats the first point at the end):
        one edge child per segment, each its own proxy; returns the first child."""
        first = None
        for a, b in zip(points[:-1], points[1:]):
            k = self._shape(body, EDGE, [a, b], vertex_radius, density, friction, restitution, filt)
            first = k if first is None else first
            self.s_owner[k] = first
        return first

    def multi(self, body, hulls, vertex_radius=float(DEFAULT_VERTEX_RADIUS), density=0.0, friction=0.2,
              restitution=0.0, filt=(1, 0xFFFF, 0, 0)) -> int:
        """MultiShapeConf with one convex hull child per point set in `hulls`
        (MultiShapeConf::AddConvexHull); returns the first child."""
        first = None
        for pts in hulls:
            k = self._shape(body, POLYGON, convex_hull(pts), vertex_radius, density, friction, restitution, filt)
            first = k if first is None else first
            self.s_owner[k] = first
        return first

    def revolute(self, a, b, anchor_a, anchor_b, ref_angle=0.0, limit=None, motor=None,
                 collide_connected=False):
        self.j_bodies.append((a, b))
        self.j_anchor.append((anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1]))
        lower, upper = limit if limit else (0.0, 0.0)
        speed, torque = motor if motor else (0.0, 0.0)
        self.j_params.append((ref_angle, lower, upper, speed, torque, 0.0))
        self.j_flags.append((1 if limit else 0, 1 if motor else 0, 1 if collide_connected else 0))
        self.j_type.append(JOINT_REVOLUTE)
        self.j_extra.append((0.0,) * 8)
        return len(self.j_bodies) - 1

    def joint(self, kind, a, b, anchor_a=(0.0, 0.0), anchor_b=(0.0, 0.0), collide_connected=False,
              enable_limit=False, enable_motor=False, **params):
        """A joint of another kind (JOINT_*) with its parameters by name (JOINT_PARAMS);
        enable_limit / enable_motor for prismatic and wheel joints.  A target joint
        has body b only: pass a=None (it is stored as a == b)."""
        names = JOINT_PARAMS[kind]
        unknown = set(params) - set(names)
        if unknown:
            raise ValueError(f"unknown parameters {sorted(unknown)} for joint kind {kind}")
        defaults = JOINT_DEFAULTS.get(kind, {})
        extra = [float(params.get(n, defaults.get(n, 0.0))) for n in names] + [0.0] * (8 - len(names))
        if kind == JOINT_TARGET:
            a = b
        self.j_bodies.append((a, b))
        self.j_anchor.append((anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1]))
        self.j_params.append((0.0,) * 6)
        self.j_flags.append((1 if enable_limit else 0, 1 if enable_motor else 0, 1 if collide_connected else 0))
        self.j_type.append(int(kind))
        self.j_extra.append(tuple(extra))
        return len(self.j_bodies) - 1

    def gear(self, joint1, joint2, ratio=1.0):
        """A gear joint coupling two earlier revolute or prismatic joints
        (GetGearJointConf, GearJointConf.cpp:66-160): its bodies A and B are the
        joints' second bodies (C and D, their first bodies, are implied)."""
        a, b = self.j_bodies[joint1][1], self.j_bodies[joint2][1]
        self.j_bodies.append((a, b))
        self.j_anchor.append((0.0, 0.0, 0.0, 0.0))
        self.j_params.append((0.0,) * 6)
        self.j_flags.append((0, 0, 0))
        self.j_type.append(JOINT_GEAR)
        self.j_extra.append((float(joint1), float(joint2), float(ratio)) + (0.0,) * 5)
        return len(self.j_bodies) - 1

    def build(self) -> Scene:
        f = lambda x, n: np.asarray(x, dtype=F32).reshape(-1, n) if n else np.asarray(x, dtype=F32)
        i = lambda x, n: np.asarray(x, dtype=np.int32).reshape(-1, n) if n else np.asarray(x, dtype=np.int32)
        return Scene(
            body_type=i(self.b_type, 0), body_pos=f(self.b_pos, 3), body_vel=f(self.b_vel, 3),
            body_acc=f(self.b_acc, 3), body_damp=f(self.b_damp, 2),
            body_flags=np.asarray(self.b_flags, dtype=np.uint32),
            shape_body=i(self.s_body, 0), shape_kind=i(self.s_kind, 0), shape_voff=i(self.s_voff, 0),
            shape_nv=i(self.s_nv, 0), shape_radius=f(self.s_radius, 0),
            shape_density=f(self.s_density, 0), shape_friction=f(self.s_friction, 0),
            shape_restitution=f(self.s_rest, 0), shape_filter=i(self.s_filter, 4),
            verts=f(self.verts, 2), joint_bodies=i(self.j_bodies, 2), joint_anchors=f(self.j_anchor, 4),
            joint_params=f(self.j_params, 6), joint_flags=i(self.j_flags, 3),
            joint_type=np.asarray(self.j_type, np.int32), joint_extra=f(self.j_extra, 8),
            shape_owner=np.asarray(self.s_owner, np.int32))


def convex_hull(points) -> list:
    """VertexSet de-duplication + gift-wrapping hull in float32 arithmetic.

    Follows ``PolygonShapeConf::Set`` (PolygonShapeConf.cpp:120-133), ``VertexSet::add``
    (VertexSet.hpp:67-108) and ``GetConvexHullAsVector`` (DistanceProxy.cpp:43-105).
    """
    min_sep2 = F32(DEFAULT_LINEAR_SLOP * DEFAULT_LINEAR_SLOP)
    pts = []
    for x, y in points:
        px, py = F32(x), F32(y)
        dup = False
        for qx, qy in pts:
            dx, dy = F32(px - qx), F32(py - qy)
            if F32(F32(F32(0) + F32(dx * dx)) + F32(dy * dy)) <= min_sep2:
                dup = True
                break
        if not dup:
            pts.append((px, py))
    n = len(pts)
    if n == 0:
        return []
    i0 = 0
    max_x = pts[0][0]
    for i in range(1, n):
        x = pts[i][0]
        if (max_x < x) or ((max_x == x) and (pts[i][1] < pts[i0][1])):
            max_x = x
            i0 = i
    hull = []
    ih = i0
    while True:
        hull.append(ih)
        ie = 0
        for j in range(1, n):
            if ie == ih:
                ie = j
                continue
            rx, ry = F32(pts[ie][0] - pts[ih][0]), F32(pts[ie][1] - pts[ih][1])
            vx, vy = F32(pts[j][0] - pts[ih][0]), F32(pts[j][1] - pts[ih][1])
            c = F32(F32(rx * vy) - F32(ry * vx))
            mv = F32(F32(F32(0) + F32(vx * vx)) + F32(vy * vy))
            mr = F32(F32(F32(0) + F32(rx * rx)) + F32(ry * ry))
            if (c < 0) or ((c == 0) and (mv > mr)):
                ie = j
        ih = ie
        if ie == i0 or len(hull) > n:
            break
    return [(float(pts[k][0]), float(pts[k][1])) for k in hull]


GRAVITY = (0.0, -10.0, 0.0)


def pyramid(rows: int = 20, x0: float = -7.0, ground_half: float = 40.0, density=1.0,
            friction=0.6, restitution=0.0) -> Scene:
    """Box pyramid on a static edge (workload 1: 20 rows, 210 boxes).

    Row i (0-based) holds rows-i unit boxes (half-extent 0.5, SetAsBox vertex
    order, which is also the hull order) at x = x0 + 0.5625 i + 1.125 j and
    y = 0.75 + 1.25 i.
    """
    ii, jj = [], []
    for i in range(rows):
        ii.extend([i] * (rows - i))
        jj.extend(range(rows - i))
    ii = np.asarray(ii, np.float64)
    jj = np.asarray(jj, np.float64)
    n = len(ii)
    nb = n + 1
    body_type = np.full(nb, DYNAMIC, np.int32)
    body_type[0] = STATIC
    pos = np.zeros((nb, 3), F32)
    pos[1:, 0] = x0 + 0.5625 * ii + 1.125 * jj
    pos[1:, 1] = 0.75 + 1.25 * ii
    acc = np.zeros((nb, 3), F32)
    acc[1:] = GRAVITY
    ns = n + 1
    box = np.asarray([(0.5, -0.5), (0.5, 0.5), (-0.5, 0.5), (-0.5, -0.5)], F32)
    verts = np.concatenate([np.asarray([(-ground_half, 0.0), (ground_half, 0.0)], F32), np.tile(box, (n, 1))])
    nv = np.full(ns, 4, np.int32)
    nv[0] = 2
    voff = np.zeros(ns, np.int32)
    voff[1:] = 2 + 4 * np.arange(n)
    kind = np.full(ns, POLYGON, np.int32)
    kind[0] = EDGE
    dens = np.full(ns, density, F32)
    dens[0] = 0.0
    filt = np.zeros((ns, 4), np.int32)
    filt[:, 0], filt[:, 1] = 1, 0xFFFF
    return Scene(body_type=body_type, body_pos=pos, body_vel=np.zeros((nb, 3), F32), body_acc=acc,
                 body_damp=np.zeros((nb, 2), F32), body_flags=np.full(nb, BF_DEFAULT, np.uint32),
                 shape_body=np.arange(ns, dtype=np.int32), shape_kind=kind, shape_voff=voff, shape_nv=nv,
                 shape_radius=np.full(ns, DEFAULT_VERTEX_RADIUS, F32), shape_density=dens,
                 shape_friction=np.full(ns, friction, F32), shape_restitution=np.full(ns, restitution, F32),
                 shape_filter=filt, verts=verts, joint_bodies=np.zeros((0, 2), np.int32),
                 joint_anchors=np.zeros((0, 4), F32), joint_params=np.zeros((0, 6), F32),
                 joint_flags=np.zeros((0, 3), np.int32))


def convex_hulls(pts: np.ndarray, counts: np.ndarray, slop: float = float(DEFAULT_LINEAR_SLOP)):
    """Vectorised ``convex_hull`` over many small point sets (float32 arithmetic).

    pts: float32 [P, M, 2]; counts: int [P].  Returns (hull points [P, M, 2], hull counts).
    Same rules as ``convex_hull``: VertexSet de-duplication, then gift wrapping from
    the lowest right-most point, counter-clockwise.
    """
    pts = np.asarray(pts, dtype=F32)
    P, M = pts.shape[:2]
    counts = np.asarray(counts)
    min_sep2 = F32(F32(slop) * F32(slop))
    keep = np.zeros((P, M), dtype=bool)
    for j in range(M):
        valid = j < counts
        dup = np.zeros(P, dtype=bool)
        for i in range(j):
            dx = pts[:, j, 0] - pts[:, i, 0]
            dy = pts[:, j, 1] - pts[:, i, 1]
            dup |= keep[:, i] & ((dx * dx + dy * dy) <= min_sep2)
        keep[:, j] = valid & ~dup
    order = np.argsort(~keep, axis=1, kind="stable")
    q = np.take_along_axis(pts, order[:, :, None], axis=1)
    n = keep.sum(axis=1)
    ar = np.arange(P)
    i0 = np.zeros(P, dtype=np.int64)
    max_x = q[:, 0, 0].copy()
    for i in range(1, M):
        x = q[:, i, 0]
        better = (i < n) & ((max_x < x) | ((max_x == x) & (q[:, i, 1] < q[ar, i0, 1])))
        i0 = np.where(better, i, i0)
        max_x = np.where(better, x, max_x)
    hull = np.zeros((P, M + 1), dtype=np.int64)
    hn = np.zeros(P, dtype=np.int64)
    done = n == 0
    ih = i0.copy()
    for _ in range(M + 1):
        act = ~done
        hull[ar[act], hn[act]] = ih[act]
        hn = hn + act
        ie = np.zeros(P, dtype=np.int64)
        for j in range(1, M):
            a = act & (j < n)
            same = a & (ie == ih)
            rest = a & ~same
            rx = q[ar, ie, 0] - q[ar, ih, 0]
            ry = q[ar, ie, 1] - q[ar, ih, 1]
            vx = q[:, j, 0] - q[ar, ih, 0]
            vy = q[:, j, 1] - q[ar, ih, 1]
            c = rx * vy - ry * vx
            mv = vx * vx + vy * vy
            mr = rx * rx + ry * ry
            take = rest & ((c < 0) | ((c == 0) & (mv > mr)))
            ie = np.where(same | take, j, ie)
        ih = np.where(act, ie, ih)
        done = done | (ie == i0) | (hn > n)
    hn = np.minimum(hn, n)
    out = np.zeros((P, M, 2), dtype=F32)
    idx = hull[:, :M]
    out[:] = np.take_along_axis(q, idx[:, :, None], axis=1)
    return out, hn


def _jittered_positions(rng, n, x0, x1, y0, y1, cell, r):
    """n non-overlapping positions (bounding radius r) on a jittered grid: each body
    takes its own cell of side `cell` >= 2 r and is placed uniformly inside it."""
    nx = max(1, int((x1 - x0) // cell))
    ny = max(1, int((y1 - y0) // cell))
    if n > nx * ny:
        raise ValueError(f"{n} bodies do not fit in {nx}x{ny} cells")
    cells = rng.choice(nx * ny, size=n, replace=False)
    cx, cy = cells % nx, cells // nx
    slack = np.maximum(0.5 * cell - r, 0.0)
    x = x0 + (cx + 0.5) * cell + rng.uniform(-1.0, 1.0, n) * slack
    y = y0 + (cy + 0.5) * cell + rng.uniform(-1.0, 1.0, n) * slack
    return x, y


def _assemble(static_edges, x, y, angle, vel, radius, is_disk, nverts, density, friction, rng,
              extra_bodies=None, joints=None, shape_filter=None, acc=GRAVITY):
    """Builds a Scene: one static ground body with edges, then one dynamic body per
    entry (disk or random convex polygon of `nverts` points on a circle)."""
    n = len(x)
    nb = 1 + n
    body_type = np.full(nb, DYNAMIC, np.int32)
    body_type[0] = STATIC
    pos = np.zeros((nb, 3), F32)
    pos[1:, 0], pos[1:, 1], pos[1:, 2] = x, y, angle
    v = np.zeros((nb, 3), F32)
    if vel is not None:
        v[1:] = vel
    a = np.zeros((nb, 3), F32)
    a[1:] = acc
    flags = np.full(nb, BF_DEFAULT, np.uint32)
    # polygons
    M = 8
    pts = np.zeros((n, M, 2), F32)
    cnt = np.where(is_disk, 1, nverts)
    poly = ~is_disk
    if poly.any():
        k = int(poly.sum())
        ang = np.sort(rng.uniform(0.0, 2.0 * math.pi, size=(k, M)), axis=1)
        mask = np.arange(M)[None, :] < nverts[poly][:, None]
        ang = np.where(mask, ang, np.inf)
        ang = np.sort(ang, axis=1)
        rr = radius[poly][:, None]
        px = np.where(mask, rr * np.cos(np.where(mask, ang, 0.0)), 0.0)
        py = np.where(mask, rr * np.sin(np.where(mask, ang, 0.0)), 0.0)
        hp, hn = convex_hulls(np.stack([px, py], -1).astype(F32), nverts[poly])
        pts[poly] = hp
        cnt = cnt.copy()
        cnt[poly] = hn
    ne = len(static_edges)
    ns = ne + n
    shape_body = np.zeros(ns, np.int32)
    shape_body[ne:] = np.arange(1, nb)
    kind = np.full(ns, EDGE, np.int32)
    kind[ne:] = np.where(is_disk, DISK, POLYGON)
    nv = np.zeros(ns, np.int32)
    nv[:ne] = 2
    nv[ne:] = cnt
    voff = np.zeros(ns, np.int32)
    voff[1:] = np.cumsum(nv)[:-1]
    verts = np.zeros((int(nv.sum()), 2), F32)
    for e, (p0, p1) in enumerate(static_edges):
        verts[2 * e] = p0
        verts[2 * e + 1] = p1
    # dynamic shape vertices, vectorised scatter
    dyn_off = voff[ne:]
    dv = np.where(is_disk[:, None, None], 0.0, pts)
    sel = np.arange(M)[None, :] < cnt[:, None]
    rows = (dyn_off[:, None] + np.arange(M)[None, :])[sel]
    verts[rows] = dv[sel]
    radius_s = np.zeros(ns, F32)
    radius_s[:ne] = DEFAULT_VERTEX_RADIUS
    radius_s[ne:] = np.where(is_disk, radius, DEFAULT_VERTEX_RADIUS)
    dens = np.zeros(ns, F32)
    dens[ne:] = density
    fr = np.full(ns, friction, F32)
    rest = np.zeros(ns, F32)
    filt = np.zeros((ns, 4), np.int32)
    filt[:, 0], filt[:, 1] = 1, 0xFFFF
    return Scene(body_type=body_type, body_pos=pos, body_vel=v, body_acc=a,
                 body_damp=np.zeros((nb, 2), F32), body_flags=flags, shape_body=shape_body,
                 shape_kind=kind, shape_voff=voff, shape_nv=nv, shape_radius=radius_s,
                 shape_density=dens, shape_friction=fr, shape_restitution=rest, shape_filter=filt,
                 verts=verts, joint_bodies=np.zeros((0, 2), np.int32), joint_anchors=np.zeros((0, 4), F32),
                 joint_params=np.zeros((0, 6), F32), joint_flags=np.zeros((0, 3), np.int32))


def large_box(n_shapes: int = 100_000, size: float = 1000.0, seed: int = 0) -> Scene:
    """Workload 2: n dynamic shapes (half disks r~U[0.05,0.5], half 3-8-gons on a circle
    of radius U[0.1,0.6]) in a square closed by 4 static edges; v~N(0,1), w~N(0,0.5),
    density U[0.5,2], friction 0.4.  Positions are uniform without overlaps
    (jittered grid of 1.3 m cells)."""
    rng = np.random.default_rng(seed)
    h = size / 2.0
    n = n_shapes
    is_disk = np.arange(n) < n // 2
    radius = np.where(is_disk, rng.uniform(0.05, 0.5, n), rng.uniform(0.1, 0.6, n))
    x, y = _jittered_positions(rng, n, -h + 0.5, h - 0.5, -h + 0.5, h - 0.5, 1.3, radius)
    vel = np.stack([rng.normal(0, 1, n), rng.normal(0, 1, n), rng.normal(0, 0.5, n)], -1)
    nverts = rng.integers(3, 9, n)
    edges = [((-h, -h), (h, -h)), ((h, -h), (h, h)), ((h, h), (-h, h)), ((-h, h), (-h, -h))]
    sc = _assemble(edges, x, y, np.zeros(n), vel, radius, is_disk, nverts,
                   rng.uniform(0.5, 2.0, len(x)), 0.4, rng)
    sc.shape_density[4:] = rng.uniform(0.5, 2.0, n).astype(F32)
    sc.shape_friction[:] = F32(0.4)
    return sc


def rebase(scene: Scene, pos_com, vel, local_center, awake=None) -> Scene:
    """The scene with each body moved to a state read back from a world: centre of
    mass position (x y angle), velocity and, when given, whether it is awake.  The
    scene stores body origins, so the local centre is rotated back out; a sleeping
    body is created asleep (BodyConf::awake false)."""
    s = Scene(**{f: getattr(scene, f) for f in scene.__dataclass_fields__})
    pos_com = np.asarray(pos_com, np.float64)
    lc = np.asarray(local_center, np.float64)
    c, sn = np.cos(pos_com[:, 2]), np.sin(pos_com[:, 2])
    org = pos_com[:, :2] - np.stack([c * lc[:, 0] - sn * lc[:, 1], sn * lc[:, 0] + c * lc[:, 1]], 1)
    s.body_pos = np.ascontiguousarray(np.concatenate([org, pos_com[:, 2:3]], 1), dtype=F32)
    s.body_vel = np.ascontiguousarray(vel, dtype=F32)
    if awake is not None:
        flags = s.body_flags.copy()
        asleep = (np.asarray(awake) == 0) & (s.body_type != STATIC)
        flags[asleep] &= ~np.uint32(BF_AWAKE)
        s.body_flags = flags
    return s


def pile(n_bodies: int, rng, friction=0.6, density=1.0, width=None) -> Scene:
    """Random pile of disks and 3-8-gons (bounding radius U[0.1,0.5]) dropped from
    heights U[1,50] m onto a static edge."""
    w = width if width is not None else max(10.0, math.sqrt(n_bodies) * 2.0)
    n = n_bodies
    is_disk = rng.integers(0, 2, n).astype(bool)
    radius = rng.uniform(0.1, 0.5, n)
    cells_needed = n / ((2 * w - 2.0) // 1.1) + 1
    top = max(50.0, 1.0 + 1.1 * cells_needed + 1.1)
    x, y = _jittered_positions(rng, n, -w + 1.0, w - 1.0, 1.0, top, 1.1, radius)
    nverts = rng.integers(3, 9, n)
    return _assemble([((-w, 0.0), (w, 0.0))], x, y, np.zeros(n), None, radius, is_disk, nverts,
                     np.full(n, density), friction, rng)


def bullets(n_bodies: int, rng, size: float = 20.0, speed=(60.0, 180.0), bullet_frac: float = 0.5,
            gravity: bool = True) -> Scene:
    """Fast disks and 3..8-gons (bounding radius U[0.1,0.4]) inside a square of side 2*size
    closed by 4 static edges, moving in random directions at U[speed] m/s (1..3 m a
    1/60 s step, more than their own size): without time-of-impact sub-stepping most
    pass through the walls.  A fraction `bullet_frac` are bullets (BodyConf::bullet),
    which also sub-step against the other moving bodies."""
    h = size
    n = n_bodies
    is_disk = rng.integers(0, 2, n).astype(bool)
    radius = rng.uniform(0.1, 0.4, n)
    x, y = _jittered_positions(rng, n, -h + 1.0, h - 1.0, -h + 1.0, h - 1.0, 1.0, radius)
    ang = rng.uniform(0.0, 2.0 * math.pi, n)
    sp = rng.uniform(speed[0], speed[1], n)
    vel = np.stack([sp * np.cos(ang), sp * np.sin(ang), rng.normal(0.0, 2.0, n)], -1)
    nverts = rng.integers(3, 9, n)
    edges = [((-h, -h), (h, -h)), ((h, -h), (h, h)), ((h, h), (-h, h)), ((-h, h), (-h, -h))]
    sc = _assemble(edges, x, y, rng.uniform(-math.pi, math.pi, n), vel, radius, is_disk, nverts,
                   np.full(n, 1.0), 0.3, rng, acc=GRAVITY if gravity else (0.0, 0.0, 0.0))
    bullet = rng.uniform(0.0, 1.0, n) < bullet_frac
    sc.body_flags[1:][bullet] |= np.uint32(BF_BULLET)
    return sc


def joint_zoo(rng, per_kind: int = 4, kinds=None, n_disks: int = 12, gravity: bool = True) -> Scene:
    """Mechanisms of every joint kind side by side above a ground edge: a static
    anchor holding a dynamic box by a distance (stiff and soft), rope, weld (rigid
    and soft), friction, motor or prismatic joint (limit, motor or both), a wheel
    on a suspension (sprung or rigid, motor on or off), two boxes on a pulley and
    a box pulled to a target point, with disks dropped on them."""
    kinds = list(kinds) if kinds is not None else [JOINT_DISTANCE, JOINT_ROPE, JOINT_WELD, JOINT_FRICTION,
                                                     JOINT_MOTOR, JOINT_PRISMATIC, JOINT_WHEEL, JOINT_PULLEY,
                                                     JOINT_TARGET]
    acc = GRAVITY if gravity else (0.0, 0.0, 0.0)
    sb = SceneBuilder()
    g = sb.body(STATIC, 0.0, 0.0)
    # a pulley's two boxes take more room than one box
    spacing = {kind: 4.0 if kind == JOINT_PULLEY else 3.0 for kind in kinds}
    width = per_kind * sum(spacing.values())
    sb.edge(g, (-width, 0.0), (width, 0.0))
    x = -width / 2.0
    for kind in kinds:
        for k in range(per_kind):
            x += spacing[kind]
            anchor = sb.body(STATIC, x, 8.0)
            hx, hy = float(rng.uniform(0.2, 0.6)), float(rng.uniform(0.2, 0.6))
            by = 8.0 - float(rng.uniform(1.0, 3.0))
            bx, ba = x + float(rng.uniform(-1.5, 1.5)), float(rng.uniform(-1, 1))
            if kind == JOINT_PULLEY:
                bx, ba = x - 1.0, 0.5 * ba
            b = sb.body(DYNAMIC, bx, by, angle=ba,
                        v=(float(rng.normal(0, 2)), float(rng.normal(0, 2)), float(rng.normal(0, 1))), acc=acc)
            soft = k % 2 == 1
            if kind == JOINT_WHEEL:
                sb.disk(b, hx, density=1.0, friction=0.5)
            else:
                sb.box(b, hx, hy, density=1.0, friction=0.5)
            if kind == JOINT_DISTANCE:
                sb.joint(kind, anchor, b, (0.0, 0.0), (hx * 0.5, 0.0), length=float(rng.uniform(1.0, 3.0)),
                         frequency=2.0 if soft else 0.0, damping_ratio=0.3 if soft else 0.0)
            elif kind == JOINT_ROPE:
                sb.joint(kind, anchor, b, (0.0, 0.0), (0.0, hy * 0.5), max_length=float(rng.uniform(1.5, 3.0)))
            elif kind == JOINT_WELD:
                sb.joint(kind, anchor, b, (0.0, -1.0), (0.0, hy), reference_angle=float(rng.uniform(-0.3, 0.3)),
                         frequency=3.0 if soft else 0.0, damping_ratio=0.5 if soft else 0.0)
            elif kind == JOINT_FRICTION:
                sb.joint(kind, anchor, b, (0.0, 0.0), (0.0, 0.0), max_force=float(rng.uniform(1.0, 20.0)),
                         max_torque=float(rng.uniform(0.5, 5.0)))
            elif kind == JOINT_MOTOR:
                sb.joint(kind, anchor, b, linear_offset_x=float(rng.uniform(-1, 1)),
                         linear_offset_y=float(rng.uniform(-3, -1)), angular_offset=float(rng.uniform(-1, 1)),
                         max_force=float(rng.uniform(20.0, 200.0)), max_torque=float(rng.uniform(5.0, 50.0)),
                         correction_factor=0.3)
            elif kind == JOINT_PRISMATIC:
                t = float(rng.uniform(0.0, math.pi))
                sb.joint(kind, anchor, b, (bx - x, by - 8.0), (0.0, 0.0), enable_limit=k % 3 != 1,
                         enable_motor=k % 3 != 0, axis_x=math.cos(t), axis_y=math.sin(t), reference_angle=ba,
                         lower=-1.0, upper=float(rng.uniform(0.5, 1.5)), motor_speed=float(rng.uniform(-2, 2)),
                         max_motor_force=float(rng.uniform(10.0, 100.0)))
            elif kind == JOINT_WHEEL:
                sb.joint(kind, anchor, b, (bx - x, by - 8.0), (0.0, 0.0), enable_motor=soft,
                         axis_x=float(rng.uniform(-0.3, 0.3)), axis_y=1.0, motor_speed=float(rng.uniform(-5, 5)),
                         max_motor_torque=float(rng.uniform(1.0, 10.0)), frequency=0.0 if k % 3 == 2 else 4.0,
                         damping_ratio=0.7)
            elif kind == JOINT_PULLEY:
                b2y = 8.0 - float(rng.uniform(1.0, 3.0))
                b2 = sb.body(DYNAMIC, x + 1.0, b2y, acc=acc)
                sb.box(b2, hy, hx, density=1.0, friction=0.5)
                ga, gb = (x - 1.0, 10.0), (x + 1.0, 10.0)
                wa = (bx - math.sin(ba) * hy, by + math.cos(ba) * hy)  # body b's anchor (0, hy) in the world
                sb.joint(kind, b, b2, (0.0, hy), (0.0, hx), collide_connected=True, ground_a_x=ga[0],
                         ground_a_y=ga[1], ground_b_x=gb[0], ground_b_y=gb[1],
                         length_a=math.hypot(wa[0] - ga[0], wa[1] - ga[1]), length_b=10.0 - (b2y + hx),
                         ratio=1.5 if soft else 1.0)
            elif kind == JOINT_TARGET:
                sb.joint(kind, None, b, anchor_b=(0.5 * hx, 0.0), target_x=x + float(rng.uniform(-1, 1)),
                         target_y=float(rng.uniform(4.0, 7.0)), max_force=float(rng.uniform(20.0, 200.0)),
                         frequency=5.0 if soft else 2.0, damping_ratio=0.7)
    for _ in range(n_disks):
        d = sb.body(DYNAMIC, float(rng.uniform(-width / 2, width / 2)), float(rng.uniform(10.0, 16.0)), acc=acc)
        sb.disk(d, float(rng.uniform(0.2, 0.5)), density=1.0, friction=0.3)
    return sb.build()


def multi_child_scene(rng, n_multi: int = 24, n_disks: int = 24) -> Scene:
    """Multi-child shapes: a static ChainShapeConf terrain (hills of 40 segments,
    each segment an edge child with its own proxy) and dynamic bodies each carrying
    one MultiShapeConf of two or three convex hulls (an L, a T, a dumbbell), with
    disks, dropped onto it."""
    sb = SceneBuilder()
    g = sb.body(STATIC, 0.0, 0.0)
    xs = np.linspace(-20.0, 20.0, 41)
    ys = 1.5 * np.sin(xs * 0.35) + 0.4 * np.sin(xs * 1.3) + rng.uniform(-0.2, 0.2, xs.size)
    sb.chain(g, [(float(x), float(y)) for x, y in zip(xs, ys)], friction=0.6)
    sb.chain(g, [(-20.0, 12.0), (-20.0, ys[0]), ], friction=0.6)  # walls
    sb.chain(g, [(20.0, ys[-1]), (20.0, 12.0)], friction=0.6)
    shapes = [
        [[(-0.6, -0.2), (0.6, -0.2), (0.6, 0.2), (-0.6, 0.2)], [(-0.6, 0.2), (-0.2, 0.2), (-0.2, 0.9), (-0.6, 0.9)]],
        [[(-0.7, 0.3), (0.7, 0.3), (0.7, 0.6), (-0.7, 0.6)], [(-0.15, -0.6), (0.15, -0.6), (0.15, 0.3), (-0.15, 0.3)]],
        [[(-0.8, -0.15), (0.8, -0.15), (0.8, 0.15), (-0.8, 0.15)], [(-1.0, -0.4), (-0.6, -0.4), (-0.6, 0.4), (-1.0, 0.4)],
         [(0.6, -0.4), (1.0, -0.4), (1.0, 0.4), (0.6, 0.4)]],
    ]
    for k in range(n_multi):
        b = sb.body(DYNAMIC, float(rng.uniform(-17.0, 17.0)), float(4.0 + 1.6 * k % 8 + rng.uniform(0.0, 0.4)),
                    angle=float(rng.uniform(-math.pi, math.pi)), acc=GRAVITY)
        sb.multi(b, shapes[k % 3], density=1.0, friction=0.5)
    for k in range(n_disks):
        b = sb.body(DYNAMIC, float(rng.uniform(-17.0, 17.0)), float(12.0 + 1.2 * k % 6 + rng.uniform(0.0, 0.4)),
                    acc=GRAVITY)
        sb.disk(b, float(rng.uniform(0.2, 0.45)), density=1.0, friction=0.4)
    return sb.build()


def sensor_scene(rng, n_bodies: int = 120) -> Scene:
    """A pile falling through sensors: static sensor zones (boxes and disks) across
    the fall, and every fifth falling body a sensor itself.  Sensors make no
    manifolds and no impulses; their touching state comes from TestOverlap
    (Distance.cpp:205-216), which is what Begin/EndContact report for them."""
    sc = pile(n_bodies, rng)
    sb = SceneBuilder.from_scene(sc)
    w = max(10.0, math.sqrt(n_bodies) * 2.0)
    for k in range(6):
        z = sb.body(STATIC, -w + (k + 0.5) * (2.0 * w / 6.0), 8.0 + 6.0 * (k % 3))
        if k % 2:
            sb.disk(z, 1.5, filt=(1, 0xFFFF, 0, 1))
        else:
            sb.box(z, 2.0, 0.6, filt=(1, 0xFFFF, 0, 1))
    out = sb.build()
    falling = np.flatnonzero(out.body_type[out.shape_body] == DYNAMIC)
    out.shape_filter[falling[::5], 3] = 1
    return out


def gear_scene(rng, pairs: int = 3, n_disks: int = 10, gravity: bool = True) -> Scene:
    """Gear trains above a ground edge: pairs of wheels on revolute joints to
    static anchors coupled by gears of ratio 1..3 (one wheel driven by a motor),
    and racks on prismatic joints coupled to a pinion's revolute joint, with
    disks dropped onto them."""
    acc = GRAVITY if gravity else (0.0, 0.0, 0.0)
    sb = SceneBuilder()
    g = sb.body(STATIC, 0.0, 0.0)
    width = 8.0 * pairs
    sb.edge(g, (-width, 0.0), (width, 0.0))
    x = -width / 2.0
    for k in range(pairs):
        x += 5.0
        r1, r2 = float(rng.uniform(0.5, 1.0)), float(rng.uniform(0.3, 0.8))
        a1, a2 = sb.body(STATIC, x, 6.0), sb.body(STATIC, x + r1 + r2 + 0.2, 6.0)
        w1 = sb.body(DYNAMIC, x, 6.0, v=(0.0, 0.0, float(rng.normal(0, 2))), acc=acc)
        sb.disk(w1, r1, density=1.0, friction=0.5)
        w2 = sb.body(DYNAMIC, x + r1 + r2 + 0.2, 6.0, acc=acc)
        sb.polygon(w2, [(r2 * math.cos(t), r2 * math.sin(t)) for t in np.linspace(0, 2 * math.pi, 7)[:-1]],
                   density=1.0, friction=0.5)
        j1 = sb.revolute(a1, w1, (0.0, 0.0), (0.0, 0.0), motor=(float(rng.uniform(-3, 3)), 50.0) if k == 0 else None)
        j2 = sb.revolute(a2, w2, (0.0, 0.0), (0.0, 0.0))
        sb.gear(j1, j2, ratio=float(rng.uniform(1.0, 3.0)))
        # rack and pinion: a box sliding on a horizontal prismatic joint under the
        # first wheel, coupled to the wheel's rotation
        rb = sb.body(DYNAMIC, x, 3.0, acc=acc)
        sb.box(rb, 1.2, 0.2, density=1.0, friction=0.5)
        ra = sb.body(STATIC, x, 3.0)
        jr = sb.joint(JOINT_PRISMATIC, ra, rb, (0.0, 0.0), (0.0, 0.0), axis_x=1.0, axis_y=0.0,
                      enable_limit=True, lower=-2.0, upper=2.0)
        sb.gear(j1, jr, ratio=float(rng.uniform(-2.0, -0.5)))
    for _ in range(n_disks):
        d = sb.body(DYNAMIC, float(rng.uniform(-width / 2, width / 2)), float(rng.uniform(8.0, 12.0)), acc=acc)
        sb.disk(d, float(rng.uniform(0.2, 0.4)), density=1.0, friction=0.3)
    return sb.build()


def batched_worlds(n_worlds: int = 4096, seed: int = 1, lo: int = 16, hi: int = 2048) -> List[Scene]:
    """Workload 3: worlds with log-uniform body counts in [lo, hi]; each is, with equal
    probability, a box pyramid with as many rows as the count allows or a pile."""
    rng = np.random.default_rng(seed)
    worlds = []
    for _ in range(n_worlds):
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        n = min(max(n, lo), hi)
        if rng.uniform() < 0.5:
            rows = int((math.isqrt(8 * n + 1) - 1) // 2)
            worlds.append(pyramid(rows=max(rows, 1), x0=-0.5625 * rows))
        else:
            worlds.append(pile(n, rng))
    return worlds


def push_worlds(n_worlds: int = 64, seed: int = 2, mu: float = 0.5, disk_v=(8.0, 0.0)) -> List[Scene]:
    """Workload 4: a controllable disk pushing 32 unit boxes on a ground with friction mu."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_worlds):
        sb = SceneBuilder()
        g = sb.body(STATIC, 0.0, 0.0)
        sb.edge(g, (-50.0, 0.0), (50.0, 0.0), friction=mu)
        d = sb.body(DYNAMIC, 2.0, 0.5, v=(disk_v[0], disk_v[1], 0.0), acc=GRAVITY)
        sb.disk(d, 0.5, density=1.0, friction=mu)
        placed = []
        while len(placed) < 32:
            x = float(rng.uniform(5.0, 25.0))
            y = float(rng.uniform(0.5, 8.0))
            if any(abs(x - px) < 1.05 and abs(y - py) < 1.05 for px, py in placed):
                continue
            placed.append((x, y))
            b = sb.body(DYNAMIC, x, y, acc=GRAVITY)
            sb.box(b, 0.5, 0.5, density=1.0, friction=mu)
        out.append(sb.build())
    return out


def chains_world(rng, n_free: int = 8000, n_chains: int = 64, links: int = 32) -> Scene:
    """Workload 5 world: free mixed shapes plus chains of 0.2x1 m boxes on revolute
    joints hanging from static anchors (chain links do not collide with each other)."""
    w = 160.0 if n_free > 1000 else 40.0
    n = n_free
    is_disk = rng.integers(0, 2, n).astype(bool)
    radius = rng.uniform(0.1, 0.5, n)
    x, y = _jittered_positions(rng, n, -w + 1.0, w - 1.0, 1.0, 61.0, 1.1, radius)
    nverts = rng.integers(3, 9, n)
    free = _assemble([((-w, 0.0), (w, 0.0))], x, y, np.zeros(n), None, radius, is_disk, nverts,
                     np.ones(n), 0.6, rng)
    # append chains with a builder (small part of the world)
    sb = SceneBuilder()
    nb0 = free.n_bodies
    top = 100.0
    for c in range(n_chains):
        ax = -w + 2.0 + (2 * w - 4.0) * (c + 0.5) / n_chains
        anchor = sb.body(STATIC, ax, top)
        prev = anchor
        for k in range(links):
            yk = top - 0.5 - 1.0 * k
            b = sb.body(DYNAMIC, ax, yk, acc=GRAVITY)
            sb.box(b, 0.1, 0.5, density=1.0, friction=0.6, filt=(2, 0xFFFD, 0, 0))
            if prev == anchor:
                sb.revolute(prev + nb0, b + nb0, (0.0, 0.0), (0.0, 0.5))
            else:
                sb.revolute(prev + nb0, b + nb0, (0.0, -0.5), (0.0, 0.5))
            prev = b
    ch = sb.build()
    vbase = free.verts.shape[0]
    return Scene(
        body_type=np.concatenate([free.body_type, ch.body_type]),
        body_pos=np.concatenate([free.body_pos, ch.body_pos]),
        body_vel=np.concatenate([free.body_vel, ch.body_vel]),
        body_acc=np.concatenate([free.body_acc, ch.body_acc]),
        body_damp=np.concatenate([free.body_damp, ch.body_damp]),
        body_flags=np.concatenate([free.body_flags, ch.body_flags]),
        shape_body=np.concatenate([free.shape_body, ch.shape_body + nb0]).astype(np.int32),
        shape_kind=np.concatenate([free.shape_kind, ch.shape_kind]),
        shape_voff=np.concatenate([free.shape_voff, ch.shape_voff + vbase]).astype(np.int32),
        shape_nv=np.concatenate([free.shape_nv, ch.shape_nv]),
        shape_radius=np.concatenate([free.shape_radius, ch.shape_radius]),
        shape_density=np.concatenate([free.shape_density, ch.shape_density]),
        shape_friction=np.concatenate([free.shape_friction, ch.shape_friction]),
        shape_restitution=np.concatenate([free.shape_restitution, ch.shape_restitution]),
        shape_filter=np.concatenate([free.shape_filter, ch.shape_filter]),
        verts=np.concatenate([free.verts, ch.verts]),
        joint_bodies=ch.joint_bodies.astype(np.int32), joint_anchors=ch.joint_anchors,
        joint_params=ch.joint_params, joint_flags=ch.joint_flags)


def scene_text(scene: Scene, conf_overrides: dict | None = None) -> str:
    """Text form read by the reference driver (hexadecimal floats, exact)."""
    out = []
    if conf_overrides:
        out.append("conf " + " ".join(f"{k} {float(v).hex()}" for k, v in conf_overrides.items()))
    hx = lambda v: float(v).hex()
    for i in range(scene.n_bodies):
        p, v, a, d = scene.body_pos[i], scene.body_vel[i], scene.body_acc[i], scene.body_damp[i]
        out.append("body %d %s %d" % (scene.body_type[i], " ".join(hx(x) for x in (*p, *v, *a, *d)),
                                       scene.body_flags[i]))
    owner = scene.shape_owner
    for s in range(scene.n_shapes):
        vo, nv = scene.shape_voff[s], scene.shape_nv[s]
        f = scene.shape_filter[s]
        head = (hx(scene.shape_radius[s]), hx(scene.shape_density[s]), hx(scene.shape_friction[s]),
                hx(scene.shape_restitution[s]))
        if owner[s] >= 0:
            if owner[s] != s:
                continue  # written with its shape's first child
            kids = [s]
            while kids[-1] + 1 < scene.n_shapes and owner[kids[-1] + 1] == s:
                kids.append(kids[-1] + 1)
            if scene.shape_kind[s] == EDGE:  # chain: the children's vertices, shared ends once
                pts = [scene.verts[scene.shape_voff[s]]] + [scene.verts[scene.shape_voff[k] + 1] for k in kids]
                out.append("chain %d %d %s %s %s %s %d %d %d %d %s" % (
                    scene.shape_body[s], len(pts), *head, f[0], f[1], f[2], f[3],
                    " ".join(hx(x) for p in pts for x in p)))
            else:  # multi: each hull's vertex count and vertices
                hulls = " ".join("%d %s" % (scene.shape_nv[k], " ".join(
                    hx(x) for x in scene.verts[scene.shape_voff[k]:scene.shape_voff[k] + scene.shape_nv[k]].reshape(-1)))
                    for k in kids)
                out.append("multi %d %d %s %s %s %s %d %d %d %d %s" % (
                    scene.shape_body[s], len(kids), *head, f[0], f[1], f[2], f[3], hulls))
            continue
        vs = " ".join(hx(x) for x in scene.verts[vo:vo + nv].reshape(-1))
        out.append("shape %d %d %d %s %s %s %s %d %d %d %d %s" % (
            scene.shape_body[s], scene.shape_kind[s], nv, *head, f[0], f[1], f[2], f[3], vs))
    for j in range(scene.n_joints):
        a, b = scene.joint_bodies[j]
        an = scene.joint_anchors[j]
        pr = scene.joint_params[j]
        fl = scene.joint_flags[j]
        kind = int(scene.joint_type[j])
        if kind != JOINT_REVOLUTE:
            out.append("jointx %d %d %d %s %d %d %d %s" % (kind, a, b, " ".join(hx(x) for x in an), fl[2], fl[0],
                                                           fl[1], " ".join(hx(x) for x in scene.joint_extra[j])))
            continue
        out.append("joint %d %d %s %d %s %s %d %s %s %d" % (
            a, b, " ".join(hx(x) for x in (*an, pr[0])), fl[0], hx(pr[1]), hx(pr[2]), fl[1],
            hx(pr[3]), hx(pr[4]), fl[2]))
    return "\n".join(out) + "\n"
