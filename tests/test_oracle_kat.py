"""Known-answer tests of the CPU oracle, transcribed from the PlayRho reference's
own tests and example output (file:line provenance on each).  CPU only."""
import math

import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes

F32 = np.float32
DEFAULT_R = float(F32(0.01))  # default vertex radius of polygons and edges (2 x linear slop)


# ---- StepConf defaults (StepConf.hpp:59-161, Settings.hpp), as the reference's
# float build computes them (values read from StepConf{} of that build).
STEPCONF_DEFAULTS = {
    "deltaTime": "0x1.111112p-6", "dtRatio": "0x1p+0", "minStillTimeToSleep": "0x1p-1",
    "linearSlop": "0x1.47ae14p-8", "angularSlop": "0x1.1df46ap-5", "regResolutionRate": "0x1.99999ap-3",
    "regMinSeparation": "-0x1.eb851ep-7", "regMinMomentum": "0x0p+0", "velocityThreshold": "0x1p+0",
    "maxTranslation": "0x1p+1", "maxRotation": "0x1.8fe3ccp+1", "maxLinearCorrection": "0x1.99999ap-3",
    "maxAngularCorrection": "0x1.1df46cp-3", "linearSleepTolerance": "0x1.47ae14p-7",
    "angularSleepTolerance": "0x1.1df46ap-5", "displaceMultiplier": "0x1p+1", "aabbExtension": "0x1.999998p-4",
    "maxCirclesRatio": "0x1.4p+3",
}


def test_stepconf_defaults():
    c = oracle.default_conf()
    for k, v in STEPCONF_DEFAULTS.items():
        assert float(F32(c[k])) == float.fromhex(v), k
    assert (c["regVelocityIters"], c["regPositionIters"], c["doWarmStart"], c["doBlocksolve"]) == (8, 3, 1, 1)


def test_gravitational_body_movement():
    # UnitTests/World.cpp:1492-1535 (World.GravitationalBodyMovement)
    a, t = F32(-10), F32(0.01)
    sb = scenes.SceneBuilder()
    sb.body(scenes.DYNAMIC, 0.0, 1.0, acc=(0.0, float(a), 0.0))
    ow = oracle.OracleWorld(sb.build())
    p0 = F32(1.0)
    for k in (1, 2):
        ow.step(deltaTime=float(t))
        b = ow.bodies()
        assert b["vel"][0, 0] == 0
        assert b["vel"][0, 1] == F32(a * F32(t * F32(k)))
        assert b["pos"][0, 0] == 0
        assert b["pos"][0, 1] == F32(p0 + F32(b["vel"][0, 1] * t))
        p0 = b["pos"][0, 1]


# ---- HelloWorld/ExpectedOutput.txt: x, y, angle of the falling disk after each
# of 60 default steps.  Lines 47-50 are where the disk lands and the reference's
# time-of-impact sub-stepping (StepConf::doToi, on by default) acts: with doToi
# every line must match; without it those four lines differ (they are checked
# against the reference's own doToi = false run, tests/golden/ref_helloworld.npz).
HELLO_Y = ("4.00 3.99 3.98 3.97 3.96 3.94 3.92 3.90 3.88 3.85 3.82 3.79 3.75 3.71 3.67 3.63 3.58 3.53 3.48 "
           "3.43 3.37 3.31 3.25 3.18 3.12 3.04 2.97 2.89 2.82 2.73 2.65 2.56 2.47 2.38 2.28 2.19 2.09 1.98 "
           "1.88 1.77 1.66 1.54 1.42 1.30 1.18 1.06 1.00 1.00 1.00 1.00 1.00 1.00 1.00 1.00 1.00 1.00 1.00 "
           "1.00 1.00 1.00").split()
TOI_LINES = {46, 47, 48, 49}


@pytest.mark.parametrize("do_toi", [0, 1])
def test_helloworld_trajectory(do_toi):
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, -10.0)
    sb.box(g, 50.0, 10.0)
    b = sb.body(scenes.DYNAMIC, 0.0, 4.0, acc=(0.0, float(F32(-9.8)), 0.0))
    sb.disk(b, 1.0)
    ow = oracle.OracleWorld(sb.build())
    for i in range(60):
        ow.step(doToi=do_toi)
        xf = ow.bodies()["xf"][1]
        line = f"{xf[0]:5.2f}{xf[1]:5.2f}{math.atan2(xf[3], xf[2]):5.2f}"
        if do_toi or i not in TOI_LINES:
            assert line == f" 0.00{float(HELLO_Y[i]):5.2f} 0.00", (i, line)


# ---- CollideShapes (UnitTests/CollideShapes.cpp)
XF0 = (0.0, 0.0, 1.0, 0.0)


def test_circle_circle_horizontal():
    # CollideShapes.cpp:57-83
    m = oracle.collide(0, [(0, 0)], 1.0, (11, -4, 1, 0), 0, [(0, 0)], 1.0, (13, -4, 1, 0))
    assert m["type"] == 1 and m["count"] == 1
    assert list(m["local_point"]) == [0, 0] and list(m["points"][0]) == [0, 0]
    assert list(m["features"][0]) == [0, 0, 0, 0]


def _box(h, w=None):
    w = h if w is None else w
    return [(w, -h), (w, h), (-w, h), (-w, -h)]


def test_identical_overlapping_squares():
    # CollideShapes.cpp:460-499
    m = oracle.collide(1, _box(1), DEFAULT_R, XF0, 1, _box(1), DEFAULT_R, XF0)
    assert m["type"] == 2 and m["count"] == 2
    assert abs(m["local_normal"][0] - 1) < 1e-5 and abs(m["local_normal"][1]) < 1e-5
    assert list(m["local_point"]) == [1, 0]
    assert list(m["points"][0]) == [-1, 1] and list(m["features"][0]) == [1, 0, 0, 2]
    assert list(m["points"][1]) == [-1, -1] and list(m["features"][1]) == [1, 0, 0, 3]


def test_horizontal_overlapping_rects():
    # CollideShapes.cpp:988-1073
    m = oracle.collide(1, _box(2), DEFAULT_R, (-2, 0, 1, 0), 1, _box(1.5, 3.0), DEFAULT_R, (2, 0, 1, 0))
    assert m["type"] == 2 and m["count"] == 2
    assert list(m["local_point"]) == [2, 0]
    assert list(m["points"][0]) == [-3.0, 1.5] and list(m["features"][0]) == [1, 0, 0, 2]
    assert list(m["points"][1]) == [-3.0, -1.5] and list(m["features"][1]) == [1, 0, 0, 3]


def test_edge_below_polygon():
    # CollideShapes.cpp:1149-1196
    m = oracle.collide(2, [(-1, 0), (1, 0)], DEFAULT_R, (0, -1, 1, 0), 1, _box(1), DEFAULT_R, XF0)
    assert m["type"] == 2 and m["count"] == 2
    assert list(m["local_point"]) == [0, 0]
    assert abs(m["local_normal"][0]) < 1e-5 and abs(m["local_normal"][1] - 1) < 1e-5
    assert list(m["points"][0]) == [-1, -1] and list(m["features"][0]) == [1, 1, 0, 3]
    assert list(m["points"][1]) == [1, -1] and list(m["features"][1]) == [1, 1, 0, 0]


def test_circle_over_right_face_of_triangle():
    # CollideShapes.cpp:351-386; the triangle's vertices in hull order start at (1,-1)
    tri = scenes.convex_hull([(-1, -1), (1, -1), (0, 1)])
    assert tri[0] == (1.0, -1.0)
    m = oracle.collide(1, tri, DEFAULT_R, XF0, 0, [(0, 0)], 1.0, (1, 1, 1, 0))
    assert m["type"] == 2 and m["count"] == 1
    assert list(m["local_point"]) == [0.5, 0.0]
    assert abs(m["local_normal"][0] - 0.894427) < 2e-4 and abs(m["local_normal"][1] - 0.44721359) < 2e-4
    assert list(m["points"][0]) == [0, 0]
    assert m["features"][0][0] == 1 and m["features"][0][2] == 0 and m["features"][0][3] == 0


# ---- GetToiViaSat (UnitTests/TimeOfImpact.cpp).  Disks are one-vertex proxies at
# the body origin; sweeps are (pos0 x y angle, pos1 x y angle, alpha0).
def _toi_limits(slop):
    s = F32(slop)
    return {"targetDepth": float(s * F32(3)), "tolerance": float(s / F32(4))}


def _toi(rA, sA, rB, sB, verts_a=((0.0, 0.0),), verts_b=((0.0, 0.0),), **conf):
    return oracle.time_of_impact(verts_a, rA, sA, (0.0, 0.0), verts_b, rB, sB, (0.0, 0.0), **conf)


def test_toi_overlapped_touching_separated():
    # TimeOfImpact.Overlapped / Touching / Separated (:157-216)
    lim = _toi_limits(0.001)
    t, state, iters, _, _ = _toi(1.0, (0, 0, 0, 0, 0, 0, 0), 1.0, (0, 0, 0, 0, 0, 0, 0), **lim)
    assert (state, t, iters) == ("overlapped", 0.0, 1)
    r = float(F32(1.0) + F32(1.5) * F32(0.001))
    t, state, iters, _, _ = _toi(r, (0, 0, 0, 0, 0, 0, 0), r, (2, 0, 0, 2, 0, 0, 0), **lim)
    assert (state, t, iters) == ("touching", 0.0, 1)
    t, state, iters, _, _ = _toi(1.0, (0, 0, 0, 0, 0, 0, 0), 1.0, (4, 0, 0, 4, 0, 0, 0), **lim)
    assert (state, t, iters) == ("separated", 1.0, 1)


def test_toi_circles_collide():
    # TimeOfImpact.CollideCirclesHorizontally (:218-240) and CollideCirclesVertically (:283-305)
    lim = _toi_limits(0.001)
    t, state, iters, _, _ = _toi(1.0, (-2, 0, 0, 0, 0, 0, 0), 1.0, (2, 0, 0, 0, 0, 0, 0), **lim)
    approx = ((F32(2) - F32(1)) + F32(lim["targetDepth"]) / F32(2)) / F32(2)
    assert state == "touching" and iters == 2
    assert abs(t - float(approx)) <= 1e-6
    t, state, iters, _, _ = _toi(1.0, (0, -20, 0, 0, 20, 0, 0), 1.0, (0, 20, 0, 0, -20, 0, 0), **lim)
    assert state == "touching" and iters == 2
    assert abs(t - 0.4750375) <= 1e-6


def test_toi_parallel_paths_do_not_collide():
    # TimeOfImpact.CirclesPassingParSepPathsDontCollide (:307-335)
    lim = _toi_limits(0.001)
    t, state, iters, _, _ = _toi(1.0, (-3, 1, 0, 3, 1, 0, 0), 1.0, (3, -1, 0, -3, -1, 0, 0), **lim)
    assert state == "separated" and iters == 7
    assert abs(t - 1.0) <= 1e-3


def test_toi_edge_circle_touchingly():
    # TimeOfImpact.CollideEdgeCircleTouchingly (:242-281), float build: 0.576901972
    conf = {"targetDepth": 0.0149999997, "tolerance": 0.0, "maxToiRootIters": 30, "maxToiIters": 20,
            "maxDistanceIters": 20}
    t, state, iters, _, _ = oracle.time_of_impact(
        ((-40.0, 0.0), (40.0, 0.0)), 0.00999999977, (0, 0, 0, 0, 0, 0, 0), (0.0, 0.0),
        ((0.0, 0.0),), 0.5, (-0.490861088, 0.49556452, 1.0125972, -0.486600876, 0.494585991, 1.00495279, 0),
        (0.0, 0.0), **conf)
    assert state == "touching" and iters == 2
    assert abs(t - 0.576901972) <= 1e-9
