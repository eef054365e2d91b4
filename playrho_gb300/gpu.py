"""ctypes binding of the C ABI in include/prgpu.h (libprgpu.so, built in-tree).

``GpuBatch`` mirrors the reference's World usage for this path: a batch is
created from scenes (CreateBody/CreateShape/Attach/CreateJoint), advanced with
``step`` (Step(World&, StepConf)) and read back with ``bodies`` / ``contacts`` /
``proxies`` (GetBody, GetContacts + GetManifold, GetTree).  There is no CPU
fallback: without the library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Sequence

import numpy as np

from .scenes import Scene

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libprgpu.so")

STATUS = {0: "OK", 1: "EINVAL", 2: "ECUDA", 3: "ECAPACITY", 4: "ETIMEOUT", 5: "ENOTREADY", 6: "ESTATE"}

CONF_FLOATS = (
    "deltaTime", "dtRatio", "minStillTimeToSleep", "linearSlop", "angularSlop",
    "regResolutionRate", "regMinSeparation", "regMinMomentum", "velocityThreshold",
    "maxTranslation", "maxRotation", "maxLinearCorrection", "maxAngularCorrection",
    "linearSleepTolerance", "angularSleepTolerance", "displaceMultiplier", "aabbExtension",
    "maxCirclesRatio")
CONF_INTS = ("regVelocityIters", "regPositionIters", "doWarmStart", "doBlocksolve")
CONF_TOI_FLOATS = ("toiResolutionRate", "toiMinSeparation", "toiMinMomentum", "targetDepth", "tolerance")
CONF_TOI_INTS = ("toiVelocityIters", "toiPositionIters", "maxToiRootIters", "maxToiIters", "maxDistanceIters",
                 "maxSubSteps", "doToi")
TOI_STATS = ("toiIslandsFound", "toiIslandsSolved", "toiContactsFound", "toiContactsAtMaxSubSteps",
             "toiContactsUpdatedToi", "toiContactsUpdatedTouching", "toiContactsSkippedTouching",
             "toiContactsAdded", "toiProxiesMoved", "toiSumPosIters", "toiSumVelIters", "toiMaxDistIters",
             "toiMaxToiIters", "toiMaxRootIters", "toiRounds")
# ToiOutput::State as prgpu_time_of_impact reports it
TOI_STATES = ("unknown", "overlapped", "touching", "separated", "maxRootIters", "nextAfter", "maxToiIters",
              "belowMinTarget", "maxDistIters", "targetDepthExceedsTotalRadius", "minTargetSquaredOverflow",
              "maxTargetSquaredOverflow")


class StepConf(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_float) for n in CONF_FLOATS] + [(n, ctypes.c_int32) for n in CONF_INTS]
                + [(n, ctypes.c_float) for n in CONF_TOI_FLOATS] + [(n, ctypes.c_int32) for n in CONF_TOI_INTS])


class StepStats(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_uint32) for n in (
        "contactsAdded", "contactsDestroyed", "contactsUpdated", "islandsFound", "islandsSolved",
        "bodiesSlept", "proxiesMoved", "sumPosIters", "liveContacts", "activeConstraints", "colours",
        "serialConstraints")] + [("minSeparation", ctypes.c_float), ("maxIncImpulse", ctypes.c_float)]
        + [(n, ctypes.c_uint32) for n in TOI_STATS]
        + [("toiMinSeparation", ctypes.c_float), ("toiMaxIncImpulse", ctypes.c_float)]
        + [("bodiesSolved", ctypes.c_uint32)])


class BatchDesc(ctypes.Structure):
    P = ctypes.c_void_p
    _fields_ = [
        ("n_worlds", ctypes.c_uint32), ("world_body_count", P), ("world_shape_count", P),
        ("world_joint_count", P), ("n_bodies", ctypes.c_uint32), ("body_type", P), ("body_pos", P),
        ("body_vel", P), ("body_acc", P), ("body_damp", P), ("body_flags", P),
        ("n_shapes", ctypes.c_uint32), ("shape_body", P), ("shape_kind", P), ("shape_voff", P),
        ("shape_nv", P), ("shape_radius", P), ("shape_density", P), ("shape_friction", P),
        ("shape_restitution", P), ("shape_filter", P), ("n_verts", ctypes.c_uint32), ("verts", P),
        ("n_joints", ctypes.c_uint32), ("joint_bodies", P), ("joint_anchors", P), ("joint_params", P),
        ("joint_flags", P), ("contact_capacity", ctypes.c_uint32), ("candidate_capacity", ctypes.c_uint32),
        ("body_mass", P), ("joint_type", P), ("joint_extra", P), ("shape_owner", P)]


class Schedule(ctypes.Structure):
    _fields_ = [("sweep_mode", ctypes.c_int32), ("warp_world_max_bodies", ctypes.c_uint32),
                ("stage_bytes", ctypes.c_uint32), ("step_ms", ctypes.c_float),
                ("group_world_max_bodies", ctypes.c_uint32)]


class PrgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"prgpu {STATUS.get(code, code)}: {msg}")
        self.code = code


_LIB = None


def load_library(path: str = LIB_PATH):
    """Loads libprgpu.so; raises if it has not been built (no silent fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise PrgpuError(5, f"{path} is missing: build it with playrho_gb300/build.py")
    lib = ctypes.CDLL(path)
    P, U, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
    lib.prgpu_abi_version.restype = I
    lib.prgpu_default_step_conf.argtypes = [ctypes.POINTER(StepConf)]
    lib.prgpu_world_create.argtypes = [ctypes.POINTER(BatchDesc), I, ctypes.POINTER(P)]
    lib.prgpu_world_destroy.argtypes = [P]
    lib.prgpu_step.argtypes = [P, ctypes.POINTER(StepConf), ctypes.POINTER(StepStats)]
    lib.prgpu_step_n.argtypes = [P, ctypes.POINTER(StepConf), I]
    lib.prgpu_step_async.argtypes = [P, ctypes.POINTER(StepConf), I]
    lib.prgpu_synchronize.argtypes = [P]
    lib.prgpu_get_counts.argtypes = [P, P, P, P, P, P]
    lib.prgpu_download_bodies.argtypes = [P, P, P, P, P, P, P]
    lib.prgpu_upload_body_states.argtypes = [P, U, U, P, P]
    lib.prgpu_download_contacts.argtypes = [P, U, P, P, P, P, P, P, P, P]
    lib.prgpu_download_contact_seq.argtypes = [P, U, P, P]
    lib.prgpu_query_aabb.argtypes = [P, U, P, U, P, P]
    lib.prgpu_download_proxies.argtypes = [P, P]
    lib.prgpu_last_error.argtypes = [P, ctypes.c_char_p, I]
    lib.prgpu_convex_hull.argtypes = [P, I, ctypes.c_float, P]
    lib.prgpu_convex_hull.restype = I
    lib.prgpu_prepare_bodies.argtypes = [ctypes.POINTER(BatchDesc), P, P, P]
    lib.prgpu_step_profiled.argtypes = [P, ctypes.POINTER(StepConf), P, I, ctypes.POINTER(StepStats)]
    lib.prgpu_last_step_phase_ms.argtypes = [P, P, I]
    lib.prgpu_graph_kernel_count.argtypes = [P, P]
    lib.prgpu_set_sweep_mode.argtypes = [P, I]
    lib.prgpu_get_sweep_mode.argtypes = [P, P]
    lib.prgpu_set_warp_world_max_bodies.argtypes = [P, U]
    lib.prgpu_get_warp_world_max_bodies.argtypes = [P, P]
    lib.prgpu_set_stage_bytes.argtypes = [P, U]
    lib.prgpu_get_stage_bytes.argtypes = [P, P]
    lib.prgpu_adjoint_begin.argtypes = [P, I]
    lib.prgpu_adjoint_forward.argtypes = [P, ctypes.POINTER(StepConf), I]
    lib.prgpu_adjoint_backward.argtypes = [P, P, P, P, P, P]
    lib.prgpu_adjoint_tangent.argtypes = [P, P, P, P, P, P]
    lib.prgpu_adjoint_info.argtypes = [P, P, P, P]
    lib.prgpu_adjoint_end.argtypes = [P]
    lib.prgpu_adjoint_profile.argtypes = [P, P, P, P]
    lib.prgpu_adjoint_trim.argtypes = []
    lib.prgpu_autotune.argtypes = [P, ctypes.POINTER(StepConf), I, ctypes.POINTER(Schedule)]
    lib.prgpu_time_of_impact.argtypes = [I, U, P, P, P, P, ctypes.POINTER(StepConf), P, P]
    lib.prgpu_get_body_steps.argtypes = [P, P]
    lib.prgpu_download_sweep_order.argtypes = [P, U, P, P]
    lib.prgpu_download_contacts_noalloc.argtypes = [P, U, P, P, P, P, P, P, P, P]
    lib.prgpu_download_contact_state.argtypes = [P, U, P, P, P]
    lib.prgpu_set_solve_records.argtypes = [P, I]
    lib.prgpu_query_aabbs.argtypes = [P, U, P, P, U, P, P]
    lib.prgpu_set_capacity_growth.argtypes = [P, I]
    lib.prgpu_get_capacities.argtypes = [P, P, P]
    lib.prgpu_set_wait_limit.argtypes = [P, U]
    lib.prgpu_set_sub_stepping.argtypes = [P, I]
    lib.prgpu_set_group_world_max_bodies.argtypes = [P, U]
    lib.prgpu_get_group_world_max_bodies.argtypes = [P, P]
    lib.prgpu_get_step_complete.argtypes = [P, U, P]
    lib.prgpu_raycast.argtypes = [P, U, P, P, P, P]
    lib.prgpu_raycast_all.argtypes = [P, U, P, U, P, P, P]
    lib.prgpu_download_solve_records.argtypes = [P, U, P, P, P, P]
    _LIB = lib
    return lib


def exported_symbols() -> List[str]:
    """The entry points this binding uses (each one declared in include/prgpu.h)."""
    return [
        "prgpu_abi_version", "prgpu_default_step_conf", "prgpu_world_create", "prgpu_world_destroy",
        "prgpu_step", "prgpu_step_n", "prgpu_step_async", "prgpu_synchronize", "prgpu_get_counts",
        "prgpu_download_bodies", "prgpu_upload_body_states", "prgpu_download_contacts",
        "prgpu_download_proxies", "prgpu_last_error", "prgpu_convex_hull", "prgpu_prepare_bodies", "prgpu_step_profiled",
        "prgpu_last_step_phase_ms", "prgpu_graph_kernel_count", "prgpu_set_sweep_mode", "prgpu_get_sweep_mode",
        "prgpu_set_warp_world_max_bodies", "prgpu_get_warp_world_max_bodies", "prgpu_autotune",
        "prgpu_set_stage_bytes", "prgpu_get_stage_bytes", "prgpu_adjoint_begin", "prgpu_adjoint_forward",
        "prgpu_adjoint_backward", "prgpu_adjoint_tangent", "prgpu_adjoint_info", "prgpu_adjoint_end",
        "prgpu_adjoint_profile", "prgpu_adjoint_trim", "prgpu_time_of_impact", "prgpu_get_body_steps",
        "prgpu_download_sweep_order", "prgpu_download_contacts_noalloc", "prgpu_download_contact_seq",
        "prgpu_query_aabb", "prgpu_download_contact_state", "prgpu_set_contact", "prgpu_set_manifold",
        "prgpu_set_solve_records", "prgpu_download_solve_records", "prgpu_query_aabbs", "prgpu_raycast",
        "prgpu_raycast_all", "prgpu_set_capacity_growth", "prgpu_get_capacities", "prgpu_set_wait_limit",
        "prgpu_set_sub_stepping", "prgpu_get_step_complete", "prgpu_set_group_world_max_bodies",
        "prgpu_get_group_world_max_bodies"]


def default_conf(**overrides) -> StepConf:
    """StepConf defaults (prgpu_default_step_conf) with the time-of-impact phase
    off unless asked for (doToi=1, the reference's own default): the regular
    phase alone is what the batch workloads and most parity checks run."""
    lib = load_library()
    c = StepConf()
    lib.prgpu_default_step_conf(ctypes.byref(c))
    c.doToi = 0
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def time_of_impact(pairs, device: int = 0, **conf):
    """GetToiViaSat on the GPU for a list of pairs ((verts_a, radius_a, sweep_a),
    (verts_b, radius_b, sweep_b)); a sweep is pos0 x y angle, pos1 x y angle,
    alpha0, local centre x y.  Returns (times, states, toi iterations, max
    distance iterations, max root iterations) as numpy arrays."""
    lib = load_library()
    nv, verts, rad, sw = [], [], [], []
    for pair in pairs:
        for v, r, s in pair:
            v = np.asarray(v, np.float32).reshape(-1, 2)
            nv.append(len(v))
            verts.append(v)
            rad.append(r)
            sw.append(np.asarray(s, np.float32).reshape(9))
    n = len(pairs)
    nv = np.asarray(nv, np.uint32)
    verts = np.ascontiguousarray(np.concatenate(verts) if verts else np.zeros((0, 2), np.float32))
    rad = np.asarray(rad, np.float32)
    sw = np.ascontiguousarray(np.stack(sw) if sw else np.zeros((0, 9), np.float32))
    t = np.zeros(n, np.float32)
    io = np.zeros((n, 4), np.int32)
    c = default_conf(**conf)
    rc = lib.prgpu_time_of_impact(device, n, nv.ctypes.data, verts.ctypes.data, rad.ctypes.data, sw.ctypes.data,
                                  ctypes.byref(c), t.ctypes.data, io.ctypes.data)
    if rc:
        raise PrgpuError(rc, "prgpu_time_of_impact failed")
    return t, io[:, 0], io[:, 1], io[:, 2], io[:, 3]


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


def _gear_offsets(scenes: Sequence[Scene], extra: np.ndarray) -> np.ndarray:
    """Gear joints name their coupled joints by index within the world; the batch
    takes global indices."""
    base = 0
    for s in scenes:
        t = np.asarray(s.joint_type).reshape(-1)
        for j in np.flatnonzero(t == 10):
            extra[base + j, 0:2] += base
        base += len(t)
    return extra


def flatten(scenes: Sequence[Scene]) -> dict:
    """World-major concatenation of scenes with global body indices."""
    body_base = np.cumsum([0] + [s.n_bodies for s in scenes])
    vert_base = np.cumsum([0] + [s.verts.shape[0] for s in scenes])
    cat = lambda f, dt: np.ascontiguousarray(np.concatenate([f(s) for s in scenes]).astype(dt))
    out = {
        "world_body_count": np.array([s.n_bodies for s in scenes], dtype=np.uint32),
        "world_shape_count": np.array([s.n_shapes for s in scenes], dtype=np.uint32),
        "world_joint_count": np.array([s.n_joints for s in scenes], dtype=np.uint32),
        "body_type": cat(lambda s: s.body_type, np.int32),
        "body_pos": cat(lambda s: s.body_pos, np.float32),
        "body_vel": cat(lambda s: s.body_vel, np.float32),
        "body_acc": cat(lambda s: s.body_acc, np.float32),
        "body_damp": cat(lambda s: s.body_damp, np.float32),
        "body_flags": cat(lambda s: s.body_flags, np.uint32),
        "shape_body": np.ascontiguousarray(np.concatenate(
            [s.shape_body + body_base[i] for i, s in enumerate(scenes)]).astype(np.uint32)),
        "shape_kind": cat(lambda s: s.shape_kind, np.int32),
        "shape_voff": np.ascontiguousarray(np.concatenate(
            [s.shape_voff + vert_base[i] for i, s in enumerate(scenes)]).astype(np.uint32)),
        "shape_nv": cat(lambda s: s.shape_nv, np.uint32),
        "shape_radius": cat(lambda s: s.shape_radius, np.float32),
        "shape_density": cat(lambda s: s.shape_density, np.float32),
        "shape_friction": cat(lambda s: s.shape_friction, np.float32),
        "shape_restitution": cat(lambda s: s.shape_restitution, np.float32),
        "shape_filter": cat(lambda s: s.shape_filter, np.int32),
        "verts": cat(lambda s: s.verts, np.float32),
        "joint_bodies": np.ascontiguousarray(np.concatenate(
            [s.joint_bodies.reshape(-1, 2) + body_base[i] for i, s in enumerate(scenes)]).astype(np.uint32)),
        "joint_anchors": cat(lambda s: s.joint_anchors.reshape(-1, 4), np.float32),
        "joint_params": cat(lambda s: s.joint_params.reshape(-1, 6), np.float32),
        "joint_flags": cat(lambda s: s.joint_flags.reshape(-1, 3), np.int32),
        "joint_type": cat(lambda s: s.joint_type.reshape(-1), np.int32),
        "joint_extra": _gear_offsets(scenes, cat(lambda s: s.joint_extra.reshape(-1, 8), np.float32)),
        # first child of a multi-child shape as a global shape index (-1 stays -1)
        "shape_owner": np.ascontiguousarray(np.concatenate(
            [np.where(s.shape_owner >= 0, s.shape_owner + shape_base_i, -1)
             for s, shape_base_i in zip(scenes, np.cumsum([0] + [x.n_shapes for x in scenes])[:-1])]
        ).astype(np.int32)),
        "body_base": body_base,
    }
    return out


def batch_desc(scenes: Sequence[Scene], contact_capacity: int = 0, candidate_capacity: int = 0):
    """The prgpu_batch_desc of a list of scenes; returns (desc, flattened arrays kept alive)."""
    f = flatten(list(scenes))
    d = BatchDesc()
    d.n_worlds = len(scenes)
    d.world_body_count = _ptr(f["world_body_count"])
    d.world_shape_count = _ptr(f["world_shape_count"])
    d.world_joint_count = _ptr(f["world_joint_count"])
    d.n_bodies = int(f["body_type"].size)
    for k in ("body_type", "body_pos", "body_vel", "body_acc", "body_damp", "body_flags", "shape_body",
              "shape_kind", "shape_voff", "shape_nv", "shape_radius", "shape_density", "shape_friction",
              "shape_restitution", "shape_filter", "verts", "joint_bodies", "joint_anchors",
              "joint_params", "joint_flags", "joint_type", "joint_extra", "shape_owner"):
        setattr(d, k, _ptr(f[k]))
    d.n_shapes = int(f["shape_body"].size)
    d.n_verts = int(f["verts"].shape[0])
    d.n_joints = int(f["joint_bodies"].shape[0])
    d.contact_capacity = contact_capacity
    d.candidate_capacity = candidate_capacity
    return d, f


def prepare_bodies(scenes: Sequence[Scene]) -> dict:
    """Host-side batch preparation (no GPU): positions, velocities and mass data."""
    lib = load_library()
    d, f = batch_desc(scenes)
    n = d.n_bodies
    pos, vel, mass = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros((n, 4), np.float32)
    rc = lib.prgpu_prepare_bodies(ctypes.byref(d), _ptr(pos), _ptr(vel), _ptr(mass))
    if rc:
        raise PrgpuError(rc, "prgpu_prepare_bodies failed")
    return {"pos": pos, "vel": vel, "inv_mass": mass[:, 0], "inv_rot_inertia": mass[:, 1], "local_center": mass[:, 2:4]}


class GpuBatch:
    """A batch of worlds on one GPU behind the C ABI."""

    def __init__(self, scenes: Sequence[Scene], device: int = 0, contact_capacity: int = 0,
                 candidate_capacity: int = 0):
        self.lib = load_library()
        self.scenes = list(scenes)
        f = flatten(self.scenes)
        self._keep = f
        d = BatchDesc()
        d.n_worlds = len(self.scenes)
        d.world_body_count = _ptr(f["world_body_count"])
        d.world_shape_count = _ptr(f["world_shape_count"])
        d.world_joint_count = _ptr(f["world_joint_count"])
        d.n_bodies = int(f["body_type"].size)
        for k in ("body_type", "body_pos", "body_vel", "body_acc", "body_damp", "body_flags", "shape_body",
                  "shape_kind", "shape_voff", "shape_nv", "shape_radius", "shape_density", "shape_friction",
                  "shape_restitution", "shape_filter", "verts", "joint_bodies", "joint_anchors",
                  "joint_params", "joint_flags", "joint_type", "joint_extra", "shape_owner"):
            setattr(d, k, _ptr(f[k]))
        d.n_shapes = int(f["shape_body"].size)
        d.n_verts = int(f["verts"].shape[0])
        d.n_joints = int(f["joint_bodies"].shape[0])
        d.contact_capacity = contact_capacity
        d.candidate_capacity = candidate_capacity
        self.n_bodies, self.n_shapes, self.n_joints = d.n_bodies, d.n_shapes, d.n_joints
        self.body_base = f["body_base"]
        self.shape_base = np.cumsum([0] + [sc.n_shapes for sc in scenes])
        h = ctypes.c_void_p()
        rc = self.lib.prgpu_world_create(ctypes.byref(d), device, ctypes.byref(h))
        if rc:
            raise PrgpuError(rc, "prgpu_world_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.prgpu_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc:
            buf = ctypes.create_string_buffer(512)
            self.lib.prgpu_last_error(self.h, buf, 512)
            raise PrgpuError(rc, f"{what}: {buf.value.decode()}")

    def step(self, conf: StepConf | None = None, **overrides) -> dict:
        c = conf if conf is not None else default_conf(**overrides)
        st = StepStats()
        self._check(self.lib.prgpu_step(self.h, ctypes.byref(c), ctypes.byref(st)), "prgpu_step")
        return {n: getattr(st, n) for n, _ in StepStats._fields_}

    def step_n(self, n: int, conf: StepConf | None = None, **overrides):
        c = conf if conf is not None else default_conf(**overrides)
        self._check(self.lib.prgpu_step_n(self.h, ctypes.byref(c), int(n)), "prgpu_step_n")

    PHASES = ("pre_contacts", "islands_colour", "constraints", "sweeps", "writeback_sleep", "sync_update",
              "find_contacts")

    def step_profiled(self, conf: StepConf | None = None, **overrides):
        """One step launched phase by phase; returns ({phase: ms}, stats)."""
        c = conf if conf is not None else default_conf(**overrides)
        ms = np.zeros(len(self.PHASES), np.float32)
        st = StepStats()
        self._check(self.lib.prgpu_step_profiled(self.h, ctypes.byref(c), _ptr(ms), len(self.PHASES),
                                                 ctypes.byref(st)), "prgpu_step_profiled")
        return dict(zip(self.PHASES, ms.tolist())), {n: getattr(st, n) for n, _ in StepStats._fields_}

    def last_step_phase_ms(self) -> dict:
        """Phase device times of the last graph-replayed step (and 'step' for all of it)."""
        ms = np.zeros(len(self.PHASES) + 1, np.float32)
        self._check(self.lib.prgpu_last_step_phase_ms(self.h, _ptr(ms), ms.size), "phase times")
        out = dict(zip(self.PHASES, ms[:-1].tolist()))
        out["step"] = float(ms[-1])
        return out

    SWEEP_MODES = {"auto": 0, "grid": 1, "per_world": 2}

    def set_sweep_mode(self, mode: str):
        """'grid' (one cooperative launch, grid barrier per colour), 'per_world'
        (one CTA per world) or 'auto'."""
        self._check(self.lib.prgpu_set_sweep_mode(self.h, self.SWEEP_MODES[mode]), "prgpu_set_sweep_mode")

    def sweep_mode(self) -> str:
        m = ctypes.c_int(0)
        self._check(self.lib.prgpu_get_sweep_mode(self.h, ctypes.byref(m)), "prgpu_get_sweep_mode")
        return {v: k for k, v in self.SWEEP_MODES.items()}[m.value]

    def set_group_world_max_bodies(self, n: int):
        """Per-world sweeps: worlds above the warp limit and of at most n bodies are
        swept by groups of 64 threads (0: no groups)."""
        self._check(self.lib.prgpu_set_group_world_max_bodies(self.h, int(n) & 0xffffffff), "group world limit")

    def group_world_max_bodies(self) -> int:
        m = ctypes.c_uint32(0)
        self._check(self.lib.prgpu_get_group_world_max_bodies(self.h, ctypes.byref(m)), "group world limit")
        return int(m.value)

    def set_warp_world_max_bodies(self, n: int):
        """Per-world sweeps: worlds of at most n bodies are swept by one warp."""
        self._check(self.lib.prgpu_set_warp_world_max_bodies(self.h, int(n) & 0xffffffff), "warp world limit")

    def warp_world_max_bodies(self) -> int:
        m = ctypes.c_uint32(0)
        self._check(self.lib.prgpu_get_warp_world_max_bodies(self.h, ctypes.byref(m)), "warp world limit")
        return int(m.value)

    def set_stage_bytes(self, n: int):
        """Shared memory for staging a world's body state in the per-world solver (0: off)."""
        self._check(self.lib.prgpu_set_stage_bytes(self.h, int(n)), "stage bytes")

    def stage_bytes(self) -> int:
        m = ctypes.c_uint32(0)
        self._check(self.lib.prgpu_get_stage_bytes(self.h, ctypes.byref(m)), "stage bytes")
        return int(m.value)

    def autotune(self, steps_per_candidate: int = 3, conf: StepConf | None = None) -> dict:
        """Times the candidate sweep schedules (advancing the world) and keeps the fastest."""
        c = conf if conf is not None else default_conf()
        sc = Schedule()
        self._check(self.lib.prgpu_autotune(self.h, ctypes.byref(c), int(steps_per_candidate), ctypes.byref(sc)),
                    "prgpu_autotune")
        inv = {v: k for k, v in self.SWEEP_MODES.items()}
        return {"sweeps": inv[sc.sweep_mode], "warp_world_max_bodies": int(sc.warp_world_max_bodies),
                "group_world_max_bodies": int(sc.group_world_max_bodies), "stage_bytes": int(sc.stage_bytes),
                "step_ms": float(sc.step_ms)}

    # ---- StepAdjoint ----
    def adjoint_begin(self, checkpoint_every: int = 16):
        """Opens a window of differentiated steps, checkpointed every k steps."""
        self._check(self.lib.prgpu_adjoint_begin(self.h, int(checkpoint_every)), "prgpu_adjoint_begin")

    def adjoint_forward(self, n: int, conf: StepConf | None = None, **overrides):
        c = conf if conf is not None else default_conf(**overrides)
        self._check(self.lib.prgpu_adjoint_forward(self.h, ctypes.byref(c), int(n)), "prgpu_adjoint_forward")

    def adjoint_backward(self, dl_dpos=None, dl_dvel=None) -> dict:
        """d(loss)/d(start state) and d(loss)/d(shape friction) from d(loss)/d(final
        centre-of-mass positions x y angle) and d(loss)/d(final velocities)."""
        n = self.n_bodies
        f32 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(n, 3)
        gp, gv = f32(dl_dpos), f32(dl_dvel)
        op, ov = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
        of = np.zeros(self.n_shapes, np.float32)
        self._check(self.lib.prgpu_adjoint_backward(self.h, _ptr(gp), _ptr(gv), _ptr(op), _ptr(ov), _ptr(of)),
                    "prgpu_adjoint_backward")
        return {"pos": op, "vel": ov, "friction": of}

    def adjoint_tangent(self, dpos=None, dvel=None, dfriction=None) -> dict:
        """FP64 forward-mode derivative of the window's final state."""
        n = self.n_bodies
        f64 = lambda a, m: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(m)
        ip, iv, iff = f64(dpos, (n, 3)), f64(dvel, (n, 3)), f64(dfriction, (self.n_shapes,))
        op, ov = np.zeros((n, 3), np.float64), np.zeros((n, 3), np.float64)
        self._check(self.lib.prgpu_adjoint_tangent(self.h, _ptr(ip), _ptr(iv), _ptr(iff), _ptr(op), _ptr(ov)),
                    "prgpu_adjoint_tangent")
        return {"pos": op, "vel": ov}

    def adjoint_info(self) -> dict:
        st, mm, ov = ctypes.c_int(), ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self.lib.prgpu_adjoint_info(self.h, ctypes.byref(st), ctypes.byref(mm), ctypes.byref(ov)),
                    "prgpu_adjoint_info")
        return {"steps": st.value, "replay_mismatches": mm.value, "tape_overflows": ov.value}

    def adjoint_profile(self) -> dict:
        f, r, v = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.prgpu_adjoint_profile(self.h, ctypes.byref(f), ctypes.byref(r), ctypes.byref(v)),
                    "prgpu_adjoint_profile")
        return {"forward_ms": f.value, "record_ms": r.value, "reverse_ms": v.value}

    def adjoint_end(self):
        self._check(self.lib.prgpu_adjoint_end(self.h), "prgpu_adjoint_end")

    def adjoint_trim(self):
        """Frees the device memory that closed adjoint windows left cached."""
        self._check(self.lib.prgpu_adjoint_trim(), "prgpu_adjoint_trim")

    def step_async(self, n: int, conf: StepConf):
        self._check(self.lib.prgpu_step_async(self.h, ctypes.byref(conf), int(n)), "prgpu_step_async")

    def synchronize(self):
        self._check(self.lib.prgpu_synchronize(self.h), "prgpu_synchronize")

    def bodies(self) -> dict:
        n = self.n_bodies
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        xf = np.zeros((n, 4), np.float32)
        mass = np.zeros((n, 4), np.float32)
        uat = np.zeros(n, np.float32)
        flags = np.zeros(n, np.uint32)
        self._check(self.lib.prgpu_download_bodies(self.h, _ptr(pos), _ptr(vel), _ptr(xf), _ptr(mass), _ptr(uat),
                                                    _ptr(flags)), "prgpu_download_bodies")
        return {"pos": pos, "vel": vel, "xf": xf, "inv_mass": mass[:, 0].copy(),
                "inv_rot_inertia": mass[:, 1].copy(), "local_center": mass[:, 2:4].copy(),
                "under_active": uat, "awake": (flags & 1).astype(np.int32)}

    def set_body_states(self, pos=None, vel=None, first: int = 0):
        pos = None if pos is None else np.ascontiguousarray(pos, dtype=np.float32)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float32)
        count = (pos if pos is not None else vel).shape[0]
        self._check(self.lib.prgpu_upload_body_states(self.h, first, count, _ptr(pos), _ptr(vel)),
                    "prgpu_upload_body_states")

    def contact_count(self) -> int:
        n = ctypes.c_uint32()
        self._check(self.lib.prgpu_get_counts(self.h, None, None, None, None, ctypes.byref(n)), "counts")
        return n.value

    def contacts(self) -> dict:
        n = self.contact_count()
        cap = max(n, 1)
        pr = np.zeros((cap, 2), np.uint32)
        bd = np.zeros((cap, 2), np.uint32)
        fl = np.zeros(cap, np.uint32)
        me = np.zeros((cap, 2), np.int32)
        hd = np.zeros((cap, 4), np.float32)
        pt = np.zeros((cap, 2, 4), np.float32)
        ft = np.zeros((cap, 2), np.uint32)
        nout = ctypes.c_uint32()
        self._check(self.lib.prgpu_download_contacts(self.h, cap, ctypes.byref(nout), _ptr(pr), _ptr(bd), _ptr(fl),
                                                      _ptr(me), _ptr(hd), _ptr(pt), _ptr(ft)), "contacts")
        n = nout.value
        feats = np.stack([(ft[:n] >> s) & 0xff for s in (0, 8, 16, 24)], axis=-1).astype(np.int32)
        return {"proxy": pr[:n].astype(np.int64), "bodies": bd[:n].astype(np.int64), "touching": (fl[:n] & 1).astype(np.int32),
                "type": me[:n, 0], "count": me[:n, 1], "local_normal": hd[:n, 0:2], "local_point": hd[:n, 2:4],
                "points": pt[:n], "features": feats}

    def query_aabb(self, world: int, aabb) -> np.ndarray:
        """World-local shape IDs whose fat AABB overlaps aabb (minx, miny, maxx, maxy)."""
        q = np.ascontiguousarray(aabb, dtype=np.float32)
        cap = int(self.shape_base[world + 1] - self.shape_base[world])
        out = np.zeros(max(cap, 1), np.uint32)
        nout = ctypes.c_uint32()
        self._check(self.lib.prgpu_query_aabb(self.h, world, _ptr(q), cap, ctypes.byref(nout), _ptr(out)), "query")
        return out[:nout.value].astype(np.int64)

    def query_aabbs(self, worlds, boxes, capacity: int = 64):
        """Many AABB queries at once (prgpu_query_aabbs): per query its overlap count
        and its world-local shape IDs (ascending)."""
        w = np.ascontiguousarray(worlds, dtype=np.uint32)
        q = np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 4)
        n = w.size
        counts = np.zeros(max(n, 1), np.uint32)
        out = np.zeros(max(n * capacity, 1), np.uint32)
        self._check(self.lib.prgpu_query_aabbs(self.h, n, _ptr(w), _ptr(q), capacity, _ptr(counts), _ptr(out)),
                    "prgpu_query_aabbs")
        return counts[:n].astype(np.int64), [out[k * capacity:k * capacity + int(counts[k])].astype(np.int64)
                                             for k in range(n)]

    def raycast(self, worlds, rays):
        """Nearest hit of each ray (prgpu_raycast): rays [n, 5] = x1 y1 x2 y2 maxFraction;
        returns shape IDs (-1: none) and hits [n, 5] = fraction, point xy, normal xy."""
        w = np.ascontiguousarray(worlds, dtype=np.uint32)
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 5)
        n = w.size
        shapes = np.zeros(max(n, 1), np.int32)
        hits = np.zeros((max(n, 1), 5), np.float32)
        self._check(self.lib.prgpu_raycast(self.h, n, _ptr(w), _ptr(r), _ptr(shapes), _ptr(hits)), "prgpu_raycast")
        return shapes[:n].astype(np.int64), hits[:n]

    def raycast_all(self, world: int, ray, capacity: int = 256) -> list:
        """Every shape one ray hits (prgpu_raycast_all), ascending by shape, as
        (shape, fraction, point x, point y, normal x, normal y)."""
        r = np.ascontiguousarray(ray, dtype=np.float32).reshape(5)
        shapes = np.zeros(capacity, np.int32)
        hits = np.zeros((capacity, 5), np.float32)
        n = ctypes.c_uint32()
        self._check(self.lib.prgpu_raycast_all(self.h, int(world), _ptr(r), capacity, ctypes.byref(n), _ptr(shapes),
                                               _ptr(hits)), "prgpu_raycast_all")
        return [(int(shapes[k]),) + tuple(hits[k]) for k in range(n.value)]

    def contact_seq(self) -> np.ndarray:
        """Creation sequence numbers of the live contacts, in the order of contacts()."""
        n = self.contact_count()
        seq = np.zeros(max(n, 1), np.uint64)
        nout = ctypes.c_uint32()
        self._check(self.lib.prgpu_download_contact_seq(self.h, seq.size, ctypes.byref(nout), _ptr(seq)), "seq")
        return seq[:nout.value]

    def body_steps(self) -> int:
        """Dynamic bodies of awake islands summed over every step run so far."""
        n = ctypes.c_uint64()
        self._check(self.lib.prgpu_get_body_steps(self.h, ctypes.byref(n)), "prgpu_get_body_steps")
        return int(n.value)

    def set_capacity_growth(self, enabled: bool = True):
        """Undo a step that runs out of contact or candidate capacity, double both and
        run it again (prgpu_set_capacity_growth)."""
        self._check(self.lib.prgpu_set_capacity_growth(self.h, int(bool(enabled))), "prgpu_set_capacity_growth")

    def capacities(self) -> tuple:
        c, k = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self.lib.prgpu_get_capacities(self.h, ctypes.byref(c), ctypes.byref(k)), "prgpu_get_capacities")
        return c.value, k.value

    def set_sub_stepping(self, enabled: bool = True):
        """SetSubStepping: each world's time-of-impact phase stops after one event."""
        self._check(self.lib.prgpu_set_sub_stepping(self.h, int(bool(enabled))), "prgpu_set_sub_stepping")

    def step_complete(self, world: int) -> bool:
        """IsStepComplete of one world."""
        v = ctypes.c_int()
        self._check(self.lib.prgpu_get_step_complete(self.h, int(world), ctypes.byref(v)), "prgpu_get_step_complete")
        return bool(v.value)

    def set_wait_limit(self, spins: int):
        """Spins a grid-barrier wait may take before it gives up (0: default)."""
        self._check(self.lib.prgpu_set_wait_limit(self.h, int(spins)), "prgpu_set_wait_limit")

    def contact_slots(self) -> np.ndarray:
        """Slot (ContactID) of every live contact, in the order of contacts()."""
        n = self.contact_count()
        out = np.zeros(max(n, 1), np.uint32)
        nout = ctypes.c_uint32()
        self._check(self.lib.prgpu_download_contact_state(self.h, out.size, ctypes.byref(nout), _ptr(out), None),
                    "contact state")
        return out[:nout.value].astype(np.int64)

    def set_solve_records(self, enabled: bool = True):
        """Keep each solved contact's impulses and iteration argument (postSolve)."""
        self._check(self.lib.prgpu_set_solve_records(self.h, int(bool(enabled))), "prgpu_set_solve_records")

    def solve_records(self) -> dict:
        """The live contacts the last step updated or solved: slot, phases (bits:
        1 pre-phase, 2 post-solve pass, 4 time-of-impact phase), solved (bool),
        point count, iteration argument, impulses (ni0 ti0 ni1 ti1)."""
        n = ctypes.c_uint32()
        self._check(self.lib.prgpu_download_solve_records(self.h, 0, ctypes.byref(n), None, None, None), "records")
        cap = max(n.value, 1)
        sl = np.zeros(cap, np.uint32)
        info = np.zeros(cap, np.uint32)
        imp = np.zeros((cap, 4), np.float32)
        self._check(self.lib.prgpu_download_solve_records(self.h, cap, ctypes.byref(n), _ptr(sl), _ptr(info), _ptr(imp)),
                    "records")
        m = n.value
        info = info[:m]
        return {"slot": sl[:m].astype(np.int64), "phases": (info & 7).astype(np.int32),
                "solved": (info & 8) != 0, "count": ((info >> 4) & 15).astype(np.int32),
                "iter": ((info >> 8) & 255).astype(np.int32), "imp": imp[:m]}

    def sweep_order(self) -> np.ndarray:
        """The last step's constraint sweep order: rows (0, shape A, shape B) for
        contacts and (1, joint, 0) for joints, global indices."""
        n = ctypes.c_uint32()
        self._check(self.lib.prgpu_download_sweep_order(self.h, 0, ctypes.byref(n), None), "sweep order")
        out = np.zeros((max(n.value, 1), 3), np.int32)
        self._check(self.lib.prgpu_download_sweep_order(self.h, n.value, ctypes.byref(n), _ptr(out)), "sweep order")
        return out[:n.value]

    def proxies(self) -> np.ndarray:
        a = np.zeros((self.n_shapes, 4), np.float32)
        self._check(self.lib.prgpu_download_proxies(self.h, _ptr(a)), "proxies")
        return a


class ContactEvents:
    """BeginContact / EndContact listener calls of each world, replayed after every
    step from two consecutive contact snapshots of a batch.

    The calls of a step come in the reference's order: first EndContact for each
    touching contact the step destroyed, in contact-list order (DestroyContacts, then
    InternalDestroy, AabbTreeWorld.cpp:2245-2331).  Then BeginContact / EndContact for
    each contact whose touching state changed, in contact-list order (UpdateContacts and
    Update, :2333-2415, 2703-2714).  The contact-list order is the creation order.
    A contact that the step created touches only if it was created at the start of the
    step, for shapes added since the last step, and was updated in that step.  Contacts
    found after the solve are not updated until the next step.  With the time-of-impact
    phase on, a contact that the phase makes
    touch and separate within one step shows only its net change.  An event is (kind,
    lower shape ID, higher shape ID) with world-local shape IDs; kind 1 is begin and 2
    is end."""

    def __init__(self, batch: "GpuBatch"):
        self.batch = batch
        self.prev = self._snapshot()

    def _snapshot(self) -> dict:
        c = self.batch.contacts()
        seq = self.batch.contact_seq()
        sb = np.asarray(self.batch.shape_base, dtype=np.int64)
        world = np.searchsorted(sb, c["proxy"][:, 0], side="right") - 1
        lo = c["proxy"].min(axis=1) - sb[world]
        hi = c["proxy"].max(axis=1) - sb[world]
        return {int(q): (int(w), int(a), int(b), int(t)) for q, w, a, b, t in
                zip(seq, world, lo, hi, c["touching"])}

    def step(self, conf=None) -> list:
        """One batch step; returns each world's listener calls of that step."""
        self.batch.step(conf)
        cur = self._snapshot()
        events = [[] for _ in range(len(self.batch.shape_base) - 1)]
        for q in sorted(self.prev):
            w, a, b, t = self.prev[q]
            if q not in cur and t:
                events[w].append((2, a, b))
        for q in sorted(cur):
            w, a, b, t = cur[q]
            if q in self.prev:
                if self.prev[q][3] != t:
                    events[w].append((1 if t else 2, a, b))
            elif t:
                events[w].append((1, a, b))
        self.prev = cur
        return events


def gpu_available() -> bool:
    try:
        import torch  # noqa: F401 -- only to ask whether a device exists

        return bool(torch.cuda.is_available())
    except Exception:
        return False
