"""The contact solver (velocity and position iterations) against the oracle with
the position solver active: bodies that interpenetrate by 2-5 cm, so that
SolvePositionConstraint (ContactSolver.cpp:494-643, PositionSolverManifold.cpp:
103-121) corrects them.

The GPU sweeps each world's constraints in graph-colour order, the reference in
island order (AabbTreeWorld.cpp:1563-1683).  Both are Gauss-Seidel orders, so the
checks are:
  * constraints that share no dynamic body (each island one contact): every order
    is the same computation, so the GPU equals the oracle in the reference's own
    order within 1e-5 relative, positions and velocities, at the default 8/3
    iterations and at 400/30;
  * coupled contacts (stacks, piles, a jointed bridge struck by bodies): the
    oracle replays the GPU's sweep order (prgpu_download_sweep_order) and the two
    agree within 1e-5 relative, positions and velocities, after one step from an
    identical state (contacts found and solved) and after the next, warm-started
    step.  That checks the arithmetic of every solver piece on coupled constraints;
  * at velocity convergence (4000 iterations) the velocities no longer depend on
    the order: one step from an identical state gives the GPU the oracle's
    velocities (reference order) within 1e-5.
    Positions after the position iterations do depend on the order even then (the
    position solver's fixed points are not unique: any state with every
    separation above -linearSlop is one), so they are checked by the replay above.
The only arithmetic that differs is sin/cos (CUDA's against the C library's).
"""
import numpy as np
import pytest

import parity_util as pu
from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch

pytestmark = pytest.mark.gpu

SKIN = 0.01  # default polygon vertex radius (PolygonShapeConf.hpp:68)


def isolated_pairs():
    """Well separated pairs, each one contact penetrating 2-5 cm: box on a static
    box (two-point face manifold), a tilted box's corner in a static box (one
    point), a disk in a static box, a box and a disk on a static edge, and two
    floating dynamic pairs (disk-disk, box-box) with no gravity."""
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, -0.5)
    sb.box(g, 4.0, 0.5, friction=0.6)
    b = sb.body(scenes.DYNAMIC, -2.0, 0.5 + 2 * SKIN - 0.03, acc=scenes.GRAVITY)
    sb.box(b, 0.5, 0.5, density=1.0, friction=0.6)
    t = sb.body(scenes.DYNAMIC, 1.5, 0.5 * np.sqrt(2.0) * np.cos(np.pi / 4 - 0.3) + SKIN - 0.04, angle=0.3,
                acc=scenes.GRAVITY)
    sb.box(t, 0.5, 0.5, density=1.0, friction=0.6)
    g2 = sb.body(scenes.STATIC, 12.0, -0.5)
    sb.box(g2, 2.0, 0.5, friction=0.6)
    d = sb.body(scenes.DYNAMIC, 12.0, 0.5 + SKIN - 0.05, acc=scenes.GRAVITY)
    sb.disk(d, 0.5, density=1.0, friction=0.6)
    e = sb.body(scenes.STATIC, 25.0, 0.0)
    sb.edge(e, (-3.0, 0.0), (3.0, 0.0), friction=0.6)
    eb = sb.body(scenes.DYNAMIC, 23.5, 0.5 + 2 * SKIN - 0.02, acc=scenes.GRAVITY)
    sb.box(eb, 0.5, 0.5, density=1.0, friction=0.6)
    ed = sb.body(scenes.DYNAMIC, 26.5, 0.4 + SKIN - 0.035, acc=scenes.GRAVITY)
    sb.disk(ed, 0.4, density=1.0, friction=0.6)
    p = sb.body(scenes.DYNAMIC, 40.0, 5.0, v=(0.3, 0.0, 0.0))
    sb.disk(p, 0.5, density=1.0, friction=0.4)
    q = sb.body(scenes.DYNAMIC, 40.0 + 1.0 - 0.03, 5.2, v=(-0.3, 0.0, 0.0))
    sb.disk(q, 0.5, density=2.0, friction=0.4)
    r = sb.body(scenes.DYNAMIC, 50.0, 5.0, angle=0.05)
    sb.box(r, 0.5, 0.5, density=1.0, friction=0.4)
    u = sb.body(scenes.DYNAMIC, 50.3, 5.0 + 1.0 + 2 * SKIN - 0.04, v=(0.0, -0.2, 0.1))
    sb.box(u, 0.5, 0.4, density=1.5, friction=0.4)
    return sb.build()


def stacks(n=5, pen=0.04, cols=3):
    """Columns of n unit boxes on a static box, each box sunk `pen` into the one
    below (two-point manifolds, block solver), columns slightly sheared."""
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, -0.5)
    sb.box(g, 20.0, 0.5, friction=0.6)
    for c in range(cols):
        for i in range(n):
            y = 0.5 + 2 * SKIN - pen + i * (1.0 + 2 * SKIN - pen)
            b = sb.body(scenes.DYNAMIC, -6.0 + 4.0 * c + 0.05 * i, y, acc=scenes.GRAVITY)
            sb.box(b, 0.5, 0.5, density=1.0, friction=0.6)
    return sb.build()


def packed_pile(pen=0.03, rows=5, per_row=8):
    """Rows of disks (and every third body a box) packed so that neighbours and
    rows overlap by `pen`, on a static edge: many coupled contacts."""
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(g, (-10.0, 0.0), (10.0, 0.0), friction=0.6)
    r = 0.5
    for row in range(rows):
        for j in range(per_row):
            x = -4.0 + j * (2 * r - pen) + (row % 2) * r
            y = r - pen + row * (np.sqrt(3) * r - pen)
            b = sb.body(scenes.DYNAMIC, x, y, acc=scenes.GRAVITY)
            if (row + j) % 3 == 0:
                sb.box(b, 0.45, 0.45, density=1.0, friction=0.6)
            else:
                sb.disk(b, r, density=1.0, friction=0.6)
    return sb.build()


def struck_chains():
    """A bridge of 8 links on revolute joints between two static anchors, with
    disks and boxes dropped onto it: joint rows and contacts in the same islands
    (links and free bodies collide; links of the bridge do not)."""
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(g, (-10.0, 0.0), (10.0, 0.0), friction=0.6)
    left = sb.body(scenes.STATIC, -4.0, 5.0)
    prev, anchor = left, (0.0, 0.0)
    for k in range(8):
        b = sb.body(scenes.DYNAMIC, -3.5 + 1.0 * k, 5.0, acc=scenes.GRAVITY)
        sb.box(b, 0.5, 0.1, density=1.0, friction=0.6, filt=(2, 0xFFFD, 0, 0))
        sb.revolute(prev, b, anchor, (-0.5, 0.0))
        prev, anchor = b, (0.5, 0.0)
    right = sb.body(scenes.STATIC, 4.0, 5.0)
    sb.revolute(prev, right, (0.5, 0.0), (0.0, 0.0))
    rng = np.random.default_rng(4)
    for i in range(10):
        b = sb.body(scenes.DYNAMIC, -3.4 + 0.75 * i + rng.uniform(-0.1, 0.1), 6.0 + 0.7 * (i % 3),
                    acc=scenes.GRAVITY)
        if i % 2:
            sb.disk(b, 0.3, density=1.0, friction=0.6)
        else:
            sb.box(b, 0.25, 0.25, density=1.0, friction=0.6)
    return sb.build()


CONFS = {
    "default": dict(),
    "converged": dict(regVelocityIters=400, regPositionIters=30, regMinSeparation=float("inf")),
}


def compare(g, o, what):
    gb, ob = g.bodies(), o.bodies()
    dp, dv = pu.rel_err(gb["pos"], ob["pos"]), pu.rel_err(gb["vel"], ob["vel"])
    assert dp <= pu.RTOL and dv <= pu.RTOL, f"{what}: relative position {dp:.3g}, velocity {dv:.3g}"


@pytest.mark.parametrize("conf", list(CONFS))
def test_isolated_contacts_reference_order(gpu_lib, conf):
    sc = isolated_pairs()
    g, o = GpuBatch([sc]), oracle.OracleWorld(sc)
    minsep = 0.0
    for k in range(6):
        st = g.step(**CONFS[conf])
        o.step(**CONFS[conf])
        compare(g, o, f"step {k + 1}")
        minsep = min(minsep, st["minSeparation"])
    assert st["activeConstraints"] >= 5
    assert minsep < -0.02  # the position solver had penetration to correct
    assert st["minSeparation"] > -0.03  # and corrected it


@pytest.mark.parametrize("conf", list(CONFS))
@pytest.mark.parametrize("scene", ["stacks", "packed_pile", "struck_chains"])
def test_coupled_contacts_in_the_gpu_sweep_order(gpu_lib, scene, conf):
    sc = {"stacks": stacks, "packed_pile": packed_pile, "struck_chains": struck_chains}[scene]()
    if scene == "struck_chains":
        # let the bodies land on the chains, then start both sides from that state
        # with identical transforms
        g0 = GpuBatch([sc])
        g0.step_n(60)
        sc = pu.rebased_worlds(g0, [sc], [0])[0]
        g = GpuBatch([sc])
        o = pu.oracle_worlds_with_gpu_transforms(g, [sc])[0]
    else:
        g, o = GpuBatch([sc]), oracle.OracleWorld(sc)
    # The first step finds the contacts and solves them (no warm start: they are
    # new); the second warm-starts from the first's impulses.  Later steps would
    # carry the first steps' sin/cos rounding forward, so the check stops there.
    steps = 2
    touched, minsep = 0, 0.0
    for k in range(steps):
        st = g.step(**CONFS[conf])
        minsep = min(minsep, st["minSeparation"])
        order = g.sweep_order()
        touched = max(touched, len(order))
        # the oracle's contacts before this step are the ones the GPU just swept
        o.set_solve_order(order)
        o.step(**CONFS[conf])
        compare(g, o, f"{scene} step {k + 1}")
    assert touched > (10 if scene != "struck_chains" else 20)
    if scene != "struck_chains":
        assert minsep < -0.02  # the position solver had penetration to correct


def frictionless_pile():
    sc = packed_pile()
    sc.shape_friction[:] = 0.0
    return sc


@pytest.mark.parametrize("scene", ["stacks", "frictionless_pile"])
def test_velocities_at_convergence_reference_order(gpu_lib, scene):
    """Where the velocity problem has one solution, the Gauss-Seidel order stops
    mattering at convergence.  Stacks of boxes (two-point manifolds, block
    solver, friction) and a packed frictionless pile have one; the packed pile
    with friction does not: its statically indeterminate friction impulses leave
    the velocities order dependent at any iteration count (0.19 m/s between two
    orders of the oracle itself after 20,000 iterations), so it is checked only
    in the replayed order above."""
    sc = stacks(n=4) if scene == "stacks" else frictionless_pile()
    conf = dict(regVelocityIters=4000, regPositionIters=30, regMinSeparation=float("inf"))
    g, o = GpuBatch([sc]), oracle.OracleWorld(sc)
    # one step from the identical initial state: the first step creates the
    # proxies, finds the contacts and solves them (a second step would start from
    # positions that the order-dependent position iterations left differently)
    st = g.step(**conf)
    o.step(**conf)
    assert st["activeConstraints"] >= 10
    dv = pu.rel_err(g.bodies()["vel"], o.bodies()["vel"])
    assert dv <= pu.RTOL, f"velocities at convergence differ by {dv:.3g}"
