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
# Body flags (BodyConf booleans): allowSleep, awake, fixedRotation, enabled.
BF_ALLOW_SLEEP, BF_AWAKE, BF_FIXED_ROTATION, BF_ENABLED = 1, 2, 4, 8
BF_DEFAULT = BF_ALLOW_SLEEP | BF_AWAKE | BF_ENABLED

DEFAULT_LINEAR_SLOP = F32(0.005)
DEFAULT_VERTEX_RADIUS = F32(DEFAULT_LINEAR_SLOP * F32(2))  # PolygonShapeConf.hpp:68


@dataclasses.dataclass
class Scene:
    """One world: bodies, shapes (one child each) and revolute joints."""

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

    def revolute(self, a, b, anchor_a, anchor_b, ref_angle=0.0, limit=None, motor=None,
                 collide_connected=False):
        self.j_bodies.append((a, b))
        self.j_anchor.append((anchor_a[0], anchor_a[1], anchor_b[0], anchor_b[1]))
        lower, upper = limit if limit else (0.0, 0.0)
        speed, torque = motor if motor else (0.0, 0.0)
        self.j_params.append((ref_angle, lower, upper, speed, torque, 0.0))
        self.j_flags.append((1 if limit else 0, 1 if motor else 0, 1 if collide_connected else 0))
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
            joint_params=f(self.j_params, 6), joint_flags=i(self.j_flags, 3))


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
            friction=0.6, restitution=0.0, builder: SceneBuilder | None = None) -> Scene:
    """Box pyramid on a static edge (workload 1: 20 rows, 210 boxes).

    Row i (0-based) holds rows-i unit boxes (half-extent 0.5) at
    x = x0 + 0.5625 i + 1.125 j and y = 0.75 + 1.25 i.
    """
    sb = builder or SceneBuilder()
    g = sb.body(STATIC, 0.0, 0.0)
    sb.edge(g, (-ground_half, 0.0), (ground_half, 0.0), friction=friction)
    for i in range(rows):
        y = 0.75 + 1.25 * i
        for j in range(rows - i):
            x = x0 + 0.5625 * i + 1.125 * j
            b = sb.body(DYNAMIC, x, y, acc=GRAVITY)
            sb.box(b, 0.5, 0.5, density=density, friction=friction, restitution=restitution)
    return sb.build() if builder is None else None


def _random_convex(rng, r, nmin=3, nmax=8):
    n = int(rng.integers(nmin, nmax + 1))
    ang = np.sort(rng.uniform(0.0, 2.0 * math.pi, size=n))
    return [(r * math.cos(a), r * math.sin(a)) for a in ang]


class _Grid:
    """Uniform-grid overlap rejection of bounding circles during scene generation."""

    def __init__(self, cell: float):
        self.cell = cell
        self.cells = {}

    def free(self, x, y, r):
        c = self.cell
        i0, i1 = int(math.floor((x - r - 0.6) / c)), int(math.floor((x + r + 0.6) / c))
        j0, j1 = int(math.floor((y - r - 0.6) / c)), int(math.floor((y + r + 0.6) / c))
        for i in range(i0, i1 + 1):
            for j in range(j0, j1 + 1):
                for (qx, qy, qr) in self.cells.get((i, j), ()):
                    if (qx - x) ** 2 + (qy - y) ** 2 < (qr + r) ** 2:
                        return False
        return True

    def add(self, x, y, r):
        k = (int(math.floor(x / self.cell)), int(math.floor(y / self.cell)))
        self.cells.setdefault(k, []).append((x, y, r))


def _add_random_shape(sb, rng, x, y, r, is_disk, density, friction, vel=None):
    v = vel if vel is not None else (0.0, 0.0, 0.0)
    b = sb.body(DYNAMIC, x, y, v=v, acc=GRAVITY)
    if is_disk:
        sb.disk(b, r, density=density, friction=friction)
    else:
        sb.polygon(b, _random_convex(rng, r), density=density, friction=friction)
    return b


def large_box(n_shapes: int = 100_000, size: float = 1000.0, seed: int = 0) -> Scene:
    """Workload 2: n dynamic shapes (half disks, half 3-8-gons) in a walled box."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder()
    h = size / 2.0
    g = sb.body(STATIC, 0.0, 0.0)
    for a, b in (((-h, -h), (h, -h)), ((h, -h), (h, h)), ((h, h), (-h, h)), ((-h, h), (-h, -h))):
        sb.edge(g, a, b, friction=0.4)
    grid = _Grid(2.0)
    placed = 0
    while placed < n_shapes:
        is_disk = placed < n_shapes // 2
        r = float(rng.uniform(0.05, 0.5)) if is_disk else float(rng.uniform(0.1, 0.6))
        x = float(rng.uniform(-h + 1.0, h - 1.0))
        y = float(rng.uniform(-h + 1.0, h - 1.0))
        if not grid.free(x, y, r):
            continue
        grid.add(x, y, r)
        vel = (float(rng.normal(0, 1)), float(rng.normal(0, 1)), float(rng.normal(0, 0.5)))
        _add_random_shape(sb, rng, x, y, r, is_disk, float(rng.uniform(0.5, 2.0)), 0.4, vel)
        placed += 1
    return sb.build()


def pile(n_bodies: int, rng, friction=0.6, density=1.0, width=None) -> Scene:
    """Random pile of disks and 3-8-gons dropped from heights U[1,50] m onto an edge."""
    sb = SceneBuilder()
    g = sb.body(STATIC, 0.0, 0.0)
    w = width if width is not None else max(10.0, math.sqrt(n_bodies) * 2.0)
    sb.edge(g, (-w, 0.0), (w, 0.0), friction=friction)
    grid = _Grid(2.0)
    placed = 0
    while placed < n_bodies:
        is_disk = bool(rng.integers(0, 2))
        r = float(rng.uniform(0.1, 0.5))
        x = float(rng.uniform(-w + 1.0, w - 1.0))
        y = float(rng.uniform(1.0, 50.0))
        if not grid.free(x, y, r):
            continue
        grid.add(x, y, r)
        _add_random_shape(sb, rng, x, y, r, is_disk, density, friction)
        placed += 1
    return sb.build()


def batched_worlds(n_worlds: int = 4096, seed: int = 1, lo: int = 16, hi: int = 2048) -> List[Scene]:
    """Workload 3: worlds with log-uniform body counts in [lo, hi]; half pyramids, half piles."""
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
    """Workload 5 world: free mixed shapes plus chains of 0.2x1 m boxes on revolute joints."""
    sb = SceneBuilder()
    w = 160.0
    g = sb.body(STATIC, 0.0, 0.0)
    sb.edge(g, (-w, 0.0), (w, 0.0), friction=0.6)
    grid = _Grid(2.0)
    placed = 0
    while placed < n_free:
        is_disk = bool(rng.integers(0, 2))
        r = float(rng.uniform(0.1, 0.5))
        x = float(rng.uniform(-w + 1.0, w - 1.0))
        y = float(rng.uniform(1.0, 60.0))
        if not grid.free(x, y, r):
            continue
        grid.add(x, y, r)
        _add_random_shape(sb, rng, x, y, r, is_disk, 1.0, 0.6)
        placed += 1
    top = 100.0
    for c in range(n_chains):
        ax = -w + 2.0 + (2 * w - 4.0) * (c + 0.5) / n_chains
        anchor = sb.body(STATIC, ax, top)
        prev = anchor
        for k in range(links):
            y = top - 0.5 - 1.0 * k
            b = sb.body(DYNAMIC, ax, y, acc=GRAVITY)
            sb.box(b, 0.1, 0.5, density=1.0, friction=0.6, filt=(2, 0xFFFD, 0, 0))
            if prev == anchor:
                sb.revolute(prev, b, (0.0, 0.0), (0.0, 0.5))
            else:
                sb.revolute(prev, b, (0.0, -0.5), (0.0, 0.5))
            prev = b
    return sb.build()


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
    for s in range(scene.n_shapes):
        vo, nv = scene.shape_voff[s], scene.shape_nv[s]
        vs = " ".join(hx(x) for x in scene.verts[vo:vo + nv].reshape(-1))
        f = scene.shape_filter[s]
        out.append("shape %d %d %d %s %s %s %s %d %d %d %d %s" % (
            scene.shape_body[s], scene.shape_kind[s], nv, hx(scene.shape_radius[s]),
            hx(scene.shape_density[s]), hx(scene.shape_friction[s]), hx(scene.shape_restitution[s]),
            f[0], f[1], f[2], f[3], vs))
    for j in range(scene.n_joints):
        a, b = scene.joint_bodies[j]
        an = scene.joint_anchors[j]
        pr = scene.joint_params[j]
        fl = scene.joint_flags[j]
        out.append("joint %d %d %s %d %s %s %d %s %s %d" % (
            a, b, " ".join(hx(x) for x in (*an, pr[0])), fl[0], hx(pr[1]), hx(pr[2]), fl[1],
            hx(pr[3]), hx(pr[4]), fl[2]))
    return "\n".join(out) + "\n"
