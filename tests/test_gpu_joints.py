"""The GPU step with distance, rope, weld, friction, motor, prismatic, wheel,
pulley and target joints against the CPU oracle (whose joints are pinned bit for
bit to the reference:
tests/test_oracle_vs_reference.py, tests/golden/ref_joint_zoo_seed7.npz).

The GPU differs from the oracle only in sin/cos, so a mechanism alone in its
world follows the oracle to within float rounding growth; joints keep their
constraints (rope and distance lengths, weld angles, prismatic and wheel axes and
limits, pulley lengths); a batch gives each world
the bits it has alone; the adjoint refuses joint kinds it does not
differentiate.  Everything goes through the C ABI.
"""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch, PrgpuError

pytestmark = pytest.mark.gpu

KINDS = {"distance": scenes.JOINT_DISTANCE, "rope": scenes.JOINT_ROPE, "weld": scenes.JOINT_WELD,
         "friction": scenes.JOINT_FRICTION, "motor": scenes.JOINT_MOTOR, "prismatic": scenes.JOINT_PRISMATIC,
         "wheel": scenes.JOINT_WHEEL, "pulley": scenes.JOINT_PULLEY, "target": scenes.JOINT_TARGET}


def single_mechanisms(kind, n, seed):
    rng = np.random.default_rng(seed)
    return [scenes.joint_zoo(rng, per_kind=2, kinds=[kind], n_disks=0) for _ in range(n)]


@pytest.mark.parametrize("name", sorted(KINDS))
def test_joint_kind_matches_oracle(gpu_lib, name):
    worlds = single_mechanisms(KINDS[name], 6, 50 + KINDS[name])
    g = GpuBatch(worlds)
    ows = [oracle.OracleWorld(w) for w in worlds]
    for step in range(60):
        g.step()
        for ow in ows:
            ow.step()
        if step in (0, 59):
            gb = g.bodies()
            for i, ow in enumerate(ows):
                base, n = int(g.body_base[i]), worlds[i].n_bodies
                ob = ow.bodies()
                # one step: within 1e-5 relative; 60 steps: rounding growth of sin/cos only
                tol = 1e-5 if step == 0 else 2e-3
                np.testing.assert_allclose(gb["pos"][base:base + n], ob["pos"], rtol=tol, atol=tol,
                                           err_msg=f"{name} world {i} step {step}")
                np.testing.assert_allclose(gb["vel"][base:base + n], ob["vel"], rtol=tol, atol=10 * tol,
                                           err_msg=f"{name} world {i} step {step}")


def _world_point(g, base, body, local):
    xf = g.bodies()["xf"]
    c, s = xf[base + body, 2], xf[base + body, 3]
    return xf[base + body, :2] + np.array([c * local[0] - s * local[1], s * local[0] + c * local[1]])


def _anchor_delta(g, w, base, j):
    a, b = (int(x) for x in w.joint_bodies[j])
    an = w.joint_anchors[j]
    return _world_point(g, base, b, an[2:4]) - _world_point(g, base, a, an[0:2])


def _anchor_distance(g, w, base, j):
    return float(np.linalg.norm(_anchor_delta(g, w, base, j)))


def _axis(g, w, base, j):
    """The joint's axis and its perpendicular in the world (localXAxisA rotated by body A)."""
    a = int(w.joint_bodies[j][0])
    e = w.joint_extra[j]
    ax = np.array([e[0], e[1]], dtype=np.float64) / np.hypot(e[0], e[1])
    xf = g.bodies()["xf"]
    c, s = xf[base + a, 2], xf[base + a, 3]
    axis = np.array([c * ax[0] - s * ax[1], s * ax[0] + c * ax[1]])
    return axis, np.array([-axis[1], axis[0]])


def test_joint_constraints_hold(gpu_lib):
    worlds = [scenes.joint_zoo(np.random.default_rng(70 + k), per_kind=3, n_disks=8) for k in range(4)]
    g = GpuBatch(worlds)
    g.step_n(120, None)
    tol = 0.1  # the position solver's corrections under impacts, in metres / radians
    for i, w in enumerate(worlds):
        base = int(g.body_base[i])
        pos = g.bodies()["pos"]
        for j in range(w.n_joints):
            kind = int(w.joint_type[j])
            if kind == scenes.JOINT_ROPE:
                assert _anchor_distance(g, w, base, j) <= float(w.joint_extra[j][0]) + tol
            elif kind == scenes.JOINT_DISTANCE and w.joint_extra[j][1] == 0.0:
                assert abs(_anchor_distance(g, w, base, j) - float(w.joint_extra[j][0])) <= tol
            elif kind == scenes.JOINT_WELD and w.joint_extra[j][1] == 0.0:
                a, b = (int(x) for x in w.joint_bodies[j])
                rel = pos[base + b, 2] - pos[base + a, 2] - float(w.joint_extra[j][0])
                assert abs(rel) <= tol
                assert _anchor_distance(g, w, base, j) <= tol
            elif kind in (scenes.JOINT_PRISMATIC, scenes.JOINT_WHEEL):
                axis, perp = _axis(g, w, base, j)
                dv = _anchor_delta(g, w, base, j)
                assert abs(float(dv @ perp)) <= tol
                if kind == scenes.JOINT_PRISMATIC and w.joint_flags[j][0]:
                    e = w.joint_extra[j]
                    assert float(e[3]) - tol <= float(dv @ axis) <= float(e[4]) + tol
            elif kind == scenes.JOINT_PULLEY:
                a, b = (int(x) for x in w.joint_bodies[j])
                e, an = w.joint_extra[j], w.joint_anchors[j]
                la = np.linalg.norm(_world_point(g, base, a, an[0:2]) - e[0:2])
                lb = np.linalg.norm(_world_point(g, base, b, an[2:4]) - e[2:4])
                assert abs((la + e[6] * lb) - (e[4] + e[6] * e[5])) <= tol


def test_joint_batch_equals_single_worlds(gpu_lib):
    worlds = [scenes.joint_zoo(np.random.default_rng(90 + k), per_kind=2, n_disks=6) for k in range(4)]
    g = GpuBatch(worlds)
    singles = [GpuBatch([w]) for w in worlds]
    g.step_n(80, None)
    for s in singles:
        s.step_n(80, None)
    gb = g.bodies()
    for i, s in enumerate(singles):
        base, n = int(g.body_base[i]), worlds[i].n_bodies
        np.testing.assert_array_equal(gb["pos"][base:base + n], s.bodies()["pos"])
        np.testing.assert_array_equal(gb["vel"][base:base + n], s.bodies()["vel"])


def test_adjoint_rejects_other_joint_kinds(gpu_lib):
    g = GpuBatch(single_mechanisms(scenes.JOINT_WELD, 1, 3))
    with pytest.raises(PrgpuError):
        g.adjoint_begin(4)


def _gear_coordinates(g, w, base):
    """Each gear's coordinate1 + ratio * coordinate2 (revolute: the angle of B
    against A less the reference angle; prismatic: the translation along the
    axis) from the GPU's bodies, as GetGearJointConf (GearJointConf.cpp:92-170) defines it."""
    b = g.bodies()
    out = []
    for j in np.flatnonzero(np.asarray(w.joint_type) == scenes.JOINT_GEAR):
        j1, j2, ratio = int(w.joint_extra[j][0]), int(w.joint_extra[j][1]), float(w.joint_extra[j][2])
        coords = []
        for jj in (j1, j2):
            a, bb = (int(x) for x in w.joint_bodies[jj])
            if int(w.joint_type[jj]) == scenes.JOINT_PRISMATIC:
                e = w.joint_extra[jj]
                ax = np.array([e[0], e[1]], np.float64) / np.hypot(e[0], e[1])
                xa, xb = b["xf"][base + a], b["xf"][base + bb]
                d = (xb[:2] + np.array([xb[2] * w.joint_anchors[jj][2] - xb[3] * w.joint_anchors[jj][3],
                                        xb[3] * w.joint_anchors[jj][2] + xb[2] * w.joint_anchors[jj][3]])) - xa[:2]
                c, s = xa[2], xa[3]
                local = np.array([c * d[0] + s * d[1], c * d[1] - s * d[0]]) - w.joint_anchors[jj][:2]
                coords.append(float(local @ ax))
            else:
                coords.append(float(b["pos"][base + bb, 2] - b["pos"][base + a, 2] - w.joint_params[jj][0]))
        out.append(coords[0] + ratio * coords[1])
    return np.array(out)


def test_gear_joint_matches_oracle(gpu_lib):
    """Gear joints (GearJointConf: revolute-revolute gear trains, one driven by a
    motor, and rack-and-pinion couplings with a prismatic joint) are 4-body
    constraint rows, coloured over all four bodies.  A gear shares its bodies
    with the two joints it couples, so the GPU's colour order and the
    reference's joint order are different Gauss-Seidel orders of one island,
    and the oracle replays the GPU's sweep order (prgpu_download_sweep_order):
      * one step from the initial state (disks dropping onto the mechanisms):
        the GPU equals the oracle (pinned bit for bit to the reference) within
        1e-5;
      * 120 steps of the mechanisms alone: within 1e-4 (the rounding of sin/cos
        carried along), and every gear keeps its coordinate combination at its
        value at creation."""
    for k in range(4):
        w = scenes.gear_scene(np.random.default_rng(60 + k))
        g, o = GpuBatch([w]), oracle.OracleWorld(w)
        g.step()
        o.set_solve_order(g.sweep_order())
        o.step()
        np.testing.assert_allclose(g.bodies()["pos"], o.bodies()["pos"], rtol=1e-5, atol=1e-5, err_msg=f"world {k}")
        np.testing.assert_allclose(g.bodies()["vel"], o.bodies()["vel"], rtol=1e-5, atol=1e-5, err_msg=f"world {k}")

    worlds = [scenes.gear_scene(np.random.default_rng(70 + k), n_disks=0) for k in range(2)]
    for w in worlds:
        g, o = GpuBatch([w]), oracle.OracleWorld(w)
        start = _gear_coordinates(g, w, 0)
        for step in range(120):
            g.step()
            o.set_solve_order(g.sweep_order())
            o.step()
            if step in (0, 59, 119):
                gb, ob = g.bodies(), o.bodies()
                np.testing.assert_allclose(gb["pos"], ob["pos"], rtol=1e-4, atol=1e-4, err_msg=f"step {step}")
                np.testing.assert_allclose(gb["vel"], ob["vel"], rtol=1e-4, atol=1e-4, err_msg=f"step {step}")
        now = _gear_coordinates(g, w, 0)
        assert np.abs(now - start).max() < 2e-2, (now, start)
