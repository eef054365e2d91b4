"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``liboracle_f32.so`` / ``liboracle_f64.so`` (built by ``oracle/Makefile``)
and runs scenes from :mod:`playrho_gb300.scenes` through the restated world step.
Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

CONF_REAL_FIELDS = (
    "deltaTime", "dtRatio", "minStillTimeToSleep", "linearSlop", "angularSlop",
    "regResolutionRate", "regMinSeparation", "regMinMomentum", "velocityThreshold",
    "maxTranslation", "maxRotation", "maxLinearCorrection", "maxAngularCorrection",
    "linearSleepTolerance", "angularSleepTolerance", "displaceMultiplier", "aabbExtension",
    "maxCirclesRatio")
CONF_INT_FIELDS = ("regVelocityIters", "regPositionIters", "doWarmStart", "doBlocksolve")
CONF_TOI_REAL_FIELDS = ("toiResolutionRate", "toiMinSeparation", "toiMinMomentum", "targetDepth", "tolerance")
CONF_TOI_INT_FIELDS = ("toiVelocityIters", "toiPositionIters", "maxToiRootIters", "maxToiIters",
                       "maxDistanceIters", "maxSubSteps", "doToi")
STATS_INT_FIELDS = (
    "preProxiesCreated", "preProxiesMoved", "preContactsDestroyed", "preContactsAdded",
    "preContactsUpdated", "regIslandsFound", "regIslandsSolved", "regContactsAdded",
    "regContactsUpdated", "regProxiesMoved", "regBodiesSlept", "regSumPosIters", "regSumVelIters")
TOI_STATS_INT_FIELDS = (
    "toiIslandsFound", "toiIslandsSolved", "toiContactsFound", "toiContactsAtMaxSubSteps",
    "toiContactsUpdatedToi", "toiContactsUpdatedTouching", "toiContactsSkippedTouching", "toiContactsAdded",
    "toiProxiesMoved", "toiSumPosIters", "toiSumVelIters", "toiMaxDistIters", "toiMaxToiIters",
    "toiMaxRootIters")
# ToiOutput::State (ToiOutput.hpp) as the oracle numbers it
TOI_STATES = ("unknown", "overlapped", "touching", "separated", "maxRootIters", "nextAfter", "maxToiIters",
              "belowMinTarget", "maxDistIters", "targetDepthExceedsTotalRadius", "minTargetSquaredOverflow",
              "maxTargetSquaredOverflow", "notFinite")


def build() -> None:
    """Compiles the oracle libraries in place (gcc, a few seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_LIBS = {}


def _lib(double: bool):
    key = bool(double)
    if key in _LIBS:
        return _LIBS[key]
    path = os.path.join(HERE, "liboracle_f64.so" if double else "liboracle_f32.so")
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    real = ctypes.c_double if double else ctypes.c_float

    class Conf(ctypes.Structure):
        _fields_ = ([(n, real) for n in CONF_REAL_FIELDS] + [(n, ctypes.c_int) for n in CONF_INT_FIELDS]
                    + [(n, real) for n in CONF_TOI_REAL_FIELDS] + [(n, ctypes.c_int) for n in CONF_TOI_INT_FIELDS])

    class Stats(ctypes.Structure):
        _fields_ = ([(n, ctypes.c_int) for n in STATS_INT_FIELDS]
                    + [("regMinSeparation", real), ("regMaxIncImpulse", real)]
                    + [(n, ctypes.c_int) for n in TOI_STATS_INT_FIELDS]
                    + [("toiMinSeparation", real), ("toiMaxIncImpulse", real)])

    P = ctypes.c_void_p
    lib.or_world_create.restype = P
    lib.or_world_destroy.argtypes = [P]
    lib.or_add_body.argtypes = [P, ctypes.c_int] + [real] * 11 + [ctypes.c_uint]
    lib.or_add_body.restype = ctypes.c_int
    lib.or_add_shape.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                 real, real, real, real, ctypes.c_uint, ctypes.c_uint, ctypes.c_int, ctypes.c_int]
    lib.or_add_shape.restype = ctypes.c_int
    lib.or_reset_mass.argtypes = [P, ctypes.c_int]
    lib.or_set_sub_stepping.argtypes = [P, ctypes.c_int]
    lib.or_is_step_complete.argtypes = [P]
    lib.or_is_step_complete.restype = ctypes.c_int
    lib.or_set_shape_owner.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.or_add_revolute.argtypes = [P, ctypes.c_int, ctypes.c_int] + [real] * 5 + [
        ctypes.c_int, real, real, ctypes.c_int, real, real, ctypes.c_int]
    lib.or_add_revolute.restype = ctypes.c_int
    lib.or_add_joint.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [real] * 4 + [ctypes.c_int,
                                                                                           ctypes.c_void_p]
    lib.or_add_joint.restype = ctypes.c_int
    lib.or_joint_enable.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.or_add_gear.argtypes = [P, ctypes.c_int, ctypes.c_int, real]
    lib.or_add_gear.restype = ctypes.c_int
    lib.or_events.argtypes = [P, ctypes.c_void_p, ctypes.c_int]
    lib.or_events.restype = ctypes.c_int
    lib.or_solve_calls.argtypes = [P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.or_solve_calls.restype = ctypes.c_int
    lib.or_raycast.argtypes = [P, real, real, real, real, real, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.or_raycast.restype = ctypes.c_int
    lib.or_default_conf.argtypes = [ctypes.POINTER(Conf)]
    lib.or_step.argtypes = [P, ctypes.POINTER(Conf), ctypes.POINTER(Stats)]
    lib.or_body_count.argtypes = [P]
    lib.or_body_count.restype = ctypes.c_int
    lib.or_get_body.argtypes = [P, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    lib.or_set_body_state.argtypes = [P, ctypes.c_int] + [real] * 6
    lib.or_set_body_xf.argtypes = [P, ctypes.c_int] + [real] * 4
    lib.or_set_solve_order.argtypes = [P, ctypes.c_int, ctypes.c_void_p]
    lib.or_contact_count.argtypes = [P]
    lib.or_contact_count.restype = ctypes.c_int
    lib.or_get_contact.argtypes = [P, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.or_proxy_count.argtypes = [P]
    lib.or_proxy_count.restype = ctypes.c_int
    lib.or_get_proxy.argtypes = [P, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.or_collide.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, real, ctypes.c_void_p,
                               ctypes.c_int, ctypes.c_int, ctypes.c_void_p, real, ctypes.c_void_p,
                               real, real, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.or_time_of_impact.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, real, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, real,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Conf), ctypes.c_void_p]
    lib.or_time_of_impact.restype = real
    lib.or_distance.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, real, ctypes.c_void_p,
                                ctypes.c_int, ctypes.c_int, ctypes.c_void_p, real, ctypes.c_void_p,
                                ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    _LIBS[key] = (lib, real, Conf, Stats)
    return _LIBS[key]


def default_conf(double: bool = False) -> dict:
    lib, real, Conf, _ = _lib(double)
    c = Conf()
    lib.or_default_conf(ctypes.byref(c))
    return {n: getattr(c, n) for n, _ in Conf._fields_}


class OracleWorld:
    """One world of the restated step, built from a :class:`Scene`."""

    def __init__(self, scene, double: bool = False):
        self.lib, self.real, self.Conf, self.Stats = _lib(double)
        self.double = double
        self.np_real = np.float64 if double else np.float32
        self.h = ctypes.c_void_p(self.lib.or_world_create())
        lib, h = self.lib, self.h
        for i in range(scene.n_bodies):
            p, v, a, d = scene.body_pos[i], scene.body_vel[i], scene.body_acc[i], scene.body_damp[i]
            lib.or_add_body(h, int(scene.body_type[i]), *(float(x) for x in (*p, *v, *a, *d)),
                            int(scene.body_flags[i]))
        for s in range(scene.n_shapes):
            vo, nv = int(scene.shape_voff[s]), int(scene.shape_nv[s])
            xy = np.ascontiguousarray(scene.verts[vo:vo + nv].reshape(-1), dtype=self.np_real)
            f = scene.shape_filter[s]
            b = int(scene.shape_body[s])
            sid = lib.or_add_shape(h, b, int(scene.shape_kind[s]), nv, xy.ctypes.data,
                                   float(scene.shape_radius[s]), float(scene.shape_density[s]),
                                   float(scene.shape_friction[s]), float(scene.shape_restitution[s]),
                                   int(f[0]), int(f[1]), int(f[2]), int(f[3]))
            own = int(scene.shape_owner[s])
            if own >= 0:  # a child of a chain (edges) or multi shape (hulls)
                lib.or_set_shape_owner(h, sid, own, 1 if int(scene.shape_kind[own]) == 2 else 2)
            if own < 0 or s + 1 == scene.n_shapes or int(scene.shape_owner[s + 1]) != own:
                lib.or_reset_mass(h, b)  # Attach(world, body, shape, resetMassData = true)
        for j in range(scene.n_joints):
            a, b = scene.joint_bodies[j]
            an, pr, fl = scene.joint_anchors[j], scene.joint_params[j], scene.joint_flags[j]
            kind = int(scene.joint_type[j])
            if kind == 10:  # gear: the two joints it couples and the ratio
                ex = scene.joint_extra[j]
                lib.or_add_gear(h, int(ex[0]), int(ex[1]), float(ex[2]))
                continue
            if kind != 0:
                ex = np.ascontiguousarray(scene.joint_extra[j], dtype=self.np_real)
                jid = lib.or_add_joint(h, kind, int(a), int(b), *(float(x) for x in an), int(fl[2]),
                                       ex.ctypes.data)
                lib.or_joint_enable(h, jid, int(fl[0]), int(fl[1]))
                continue
            lib.or_add_revolute(h, int(a), int(b), *(float(x) for x in an), float(pr[0]), int(fl[0]),
                                float(pr[1]), float(pr[2]), int(fl[1]), float(pr[3]), float(pr[4]),
                                int(fl[2]))
        self.n_bodies = scene.n_bodies

    def __del__(self):
        try:
            self.lib.or_world_destroy(self.h)
        except Exception:
            pass

    def make_conf(self, **overrides):
        c = self.Conf()
        self.lib.or_default_conf(ctypes.byref(c))
        for k, v in overrides.items():
            setattr(c, k, v)
        return c

    def step(self, conf=None, **overrides):
        c = conf if conf is not None else self.make_conf(**overrides)
        st = self.Stats()
        self.lib.or_step(self.h, ctypes.byref(c), ctypes.byref(st))
        return {n: getattr(st, n) for n, _ in self.Stats._fields_}

    def bodies(self) -> dict:
        n = self.lib.or_body_count(self.h)
        out = np.zeros((n, 13), dtype=self.np_real)
        awake = np.zeros(n, dtype=np.int32)
        aw = ctypes.c_int()
        for i in range(n):
            self.lib.or_get_body(self.h, i, out[i].ctypes.data, ctypes.byref(aw))
            awake[i] = aw.value
        return {"pos": out[:, 0:3].copy(), "vel": out[:, 3:6].copy(), "xf": out[:, 6:10].copy(),
                "inv_mass": out[:, 10].copy(), "inv_rot_inertia": out[:, 11].copy(),
                "under_active": out[:, 12].copy(), "awake": awake}

    def set_body_state(self, i, pos, vel):
        self.lib.or_set_body_state(self.h, int(i), *(float(x) for x in (*pos, *vel)))

    def set_body_xf(self, xf4):
        """Gives every body the transformation (p.x, p.y, cos, sin) in xf4 [n, 4]
        (identical transforms on both sides of a parity check)."""
        for i, x in enumerate(np.asarray(xf4)):
            self.lib.or_set_body_xf(self.h, int(i), *(float(v) for v in x))

    def set_solve_order(self, items):
        """Solve constraints in the order of ``items`` [n, 3] from the next step on:
        (0, shape A, shape B) for a contact, (1, joint, 0) for a joint; None or an
        empty list restores the reference's order."""
        a = np.ascontiguousarray(np.asarray(items if items is not None else [], dtype=np.int32).reshape(-1, 3))
        self.lib.or_set_solve_order(self.h, int(a.shape[0]), a.ctypes.data if a.size else None)

    def events(self) -> list:
        """BeginContact (1) / EndContact (2) listener calls of the last step, in call
        order, as (kind, lower shape ID, higher shape ID)."""
        n = self.lib.or_events(self.h, None, 0)
        buf = np.zeros(max(3 * n, 3), np.int32)
        self.lib.or_events(self.h, buf.ctypes.data, n)
        return [tuple(int(x) for x in buf[3 * i:3 * i + 3]) for i in range(n)]

    def solve_calls(self) -> list:
        """PreSolveContact (3) / PostSolveContact (4) listener calls of the last step,
        in call order, as (kind, lower shape ID, higher shape ID, point count,
        iteration, ni0, ti0, ni1, ti1): preSolve's manifold before the update (the
        iteration is 0), postSolve's velocity-constraint impulses and its
        iteration argument (255: not solved)."""
        n = self.lib.or_solve_calls(self.h, None, None, 0)
        ints = np.zeros(max(5 * n, 5), np.int32)
        imp = np.zeros(max(4 * n, 4), np.float64)
        self.lib.or_solve_calls(self.h, ints.ctypes.data, imp.ctypes.data, n)
        return [tuple(int(x) for x in ints[5 * i:5 * i + 5]) + tuple(float(x) for x in imp[4 * i:4 * i + 4])
                for i in range(n)]

    def set_sub_stepping(self, flag: bool = True):
        """SetSubStepping: the time-of-impact phase stops after one event a step."""
        self.lib.or_set_sub_stepping(self.h, int(bool(flag)))

    def is_step_complete(self) -> bool:
        return bool(self.lib.or_is_step_complete(self.h))

    def raycast(self, p1, p2, max_fraction=1.0) -> list:
        """RayCast of the world with a callback that answers ResetRay: every shape
        hit, in shape order, as (shape, fraction, point x, point y, normal x, normal y)."""
        n = self.lib.or_raycast(self.h, *(float(v) for v in (p1[0], p1[1], p2[0], p2[1], max_fraction)), 0, None, None)
        shapes = np.zeros(max(n, 1), np.int32)
        hits = np.zeros((max(n, 1), 5), self.np_real)
        self.lib.or_raycast(self.h, *(float(v) for v in (p1[0], p1[1], p2[0], p2[1], max_fraction)), n,
                            shapes.ctypes.data, hits.ctypes.data)
        return [(int(shapes[k]),) + tuple(hits[k]) for k in range(n)]

    def contacts(self) -> dict:
        n = self.lib.or_contact_count(self.h)
        io = np.zeros((n, 12), dtype=np.int32)
        fo = np.zeros((n, 12), dtype=self.np_real)
        ft = np.zeros((n, 8), dtype=np.int32)
        for k in range(n):
            self.lib.or_get_contact(self.h, k, io[k].ctypes.data, fo[k].ctypes.data, ft[k].ctypes.data)
        return {"id": io[:, 0], "proxy": io[:, 1:3], "bsc_a": io[:, 3:6], "bsc_b": io[:, 6:9],
                "touching": io[:, 9], "type": io[:, 10], "count": io[:, 11], "local_normal": fo[:, 0:2],
                "local_point": fo[:, 2:4], "points": fo[:, 4:12].reshape(n, 2, 4), "features": ft.reshape(n, 2, 4)}

    def proxies(self) -> dict:
        n = self.lib.or_proxy_count(self.h)
        bsc = np.zeros((n, 3), dtype=np.int32)
        aabb = np.zeros((n, 4), dtype=self.np_real)
        for p in range(n):
            self.lib.or_get_proxy(self.h, p, bsc[p].ctypes.data, aabb[p].ctypes.data)
        return {"bsc": bsc, "aabb": aabb}


def collide(kind_a, verts_a, r_a, xf_a, kind_b, verts_b, r_b, xf_b, linear_slop=0.005,
            max_circles_ratio=10.0, double=False):
    """Stand-alone CollideShapes of the oracle for known-answer tests."""
    lib, real, _, _ = _lib(double)
    npr = np.float64 if double else np.float32
    va = np.ascontiguousarray(np.asarray(verts_a, dtype=npr).reshape(-1))
    vb = np.ascontiguousarray(np.asarray(verts_b, dtype=npr).reshape(-1))
    xa = np.ascontiguousarray(np.asarray(xf_a, dtype=npr))
    xb = np.ascontiguousarray(np.asarray(xf_b, dtype=npr))
    tc = np.zeros(2, dtype=np.int32)
    ft = np.zeros(8, dtype=np.int32)
    fo = np.zeros(8, dtype=npr)
    lib.or_collide(kind_a, va.size // 2, va.ctypes.data, r_a, xa.ctypes.data, kind_b, vb.size // 2,
                   vb.ctypes.data, r_b, xb.ctypes.data, linear_slop, max_circles_ratio,
                   tc.ctypes.data, ft.ctypes.data, fo.ctypes.data)
    return {"type": int(tc[0]), "count": int(tc[1]), "features": ft.reshape(2, 4),
            "local_normal": fo[0:2], "local_point": fo[2:4], "points": fo[4:8].reshape(2, 2)}


def time_of_impact(verts_a, r_a, sweep_a, lc_a, verts_b, r_b, sweep_b, lc_b, double=False, **conf):
    """Stand-alone GetToiViaSat of the oracle: sweeps are (pos0 xy angle, pos1 xy angle,
    alpha0); returns (time, state name, toi iterations, max distance iterations,
    max root iterations)."""
    lib, real, Conf, _ = _lib(double)
    npr = np.float64 if double else np.float32
    c = Conf()
    lib.or_default_conf(ctypes.byref(c))
    for k, v in conf.items():
        setattr(c, k, v)
    arr = lambda x: np.ascontiguousarray(np.asarray(x, dtype=npr).reshape(-1))
    va, vb, sa, sb, la, lb = (arr(x) for x in (verts_a, verts_b, sweep_a, sweep_b, lc_a, lc_b))
    io = np.zeros(4, dtype=np.int32)
    t = lib.or_time_of_impact(0, va.size // 2, va.ctypes.data, r_a, sa.ctypes.data, la.ctypes.data,
                              0, vb.size // 2, vb.ctypes.data, r_b, sb.ctypes.data, lb.ctypes.data,
                              ctypes.byref(c), io.ctypes.data)
    return float(t), TOI_STATES[int(io[0])], int(io[1]), int(io[2]), int(io[3])


def distance(verts_a, r_a, xf_a, verts_b, r_b, xf_b, max_iters=20, double=False):
    """Stand-alone GJK Distance of the oracle from an empty cache: (state, iterations,
    simplex size, witness point A, witness point B)."""
    lib, real, _, _ = _lib(double)
    npr = np.float64 if double else np.float32
    arr = lambda x: np.ascontiguousarray(np.asarray(x, dtype=npr).reshape(-1))
    va, vb, xa, xb = (arr(x) for x in (verts_a, verts_b, xf_a, xf_b))
    io = np.zeros(3, dtype=np.int32)
    fo = np.zeros(4, dtype=npr)
    lib.or_distance(0, va.size // 2, va.ctypes.data, r_a, xa.ctypes.data, 0, vb.size // 2, vb.ctypes.data, r_b,
                    xb.ctypes.data, max_iters, io.ctypes.data, fo.ctypes.data)
    return int(io[0]), int(io[1]), int(io[2]), fo[0:2].copy(), fo[2:4].copy()
