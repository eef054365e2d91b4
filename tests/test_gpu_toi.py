"""The GPU time-of-impact phase (StepConf::doToi) against the CPU oracle.

The oracle's TOI phase is pinned bit for bit to the reference (fixtures
tests/golden/ref_toi_*.npz, tests/test_oracle_vs_reference.py).  Here:
  * GetToiViaSat on the GPU (prgpu_time_of_impact) against the oracle's, on the
    reference's own known answers and on random pairs: bit-exact where no sweep
    rotates (the only arithmetic that differs is sin/cos), else within 1e-4;
  * whole steps with doToi on: bit-exact against the oracle where every island
    is one contact and nothing rotates (HelloWorld, frictionless bullet disks
    fired at the ground); on fast mixed shapes in a closed box, almost every
    body passes through the walls without doToi and, with it, about as few as
    in the oracle (its sub-step limit lets a handful through);
  * a batch of worlds gives each world the bits it has alone.
Everything goes through the C ABI (libprgpu.so).
"""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import gpu, scenes
from playrho_gb300.gpu import GpuBatch

pytestmark = pytest.mark.gpu

F32 = np.float32


def _sweep(p0, p1, a0=0.0, lc=(0.0, 0.0)):
    return (*p0, *p1, a0, *lc)


def test_toi_known_answers(gpu_lib):
    # UnitTests/TimeOfImpact.cpp: Overlapped, Touching, Separated, CollideCirclesHorizontally,
    # CollideCirclesVertically, CirclesPassingParSepPathsDontCollide (slop 0.001)
    s = F32(0.001)
    lim = {"targetDepth": float(s * F32(3)), "tolerance": float(s / F32(4))}
    r_touch = float(F32(1.0) + F32(1.5) * s)
    o = ((0.0, 0.0),)
    pairs = [
        ((o, 1.0, _sweep((0, 0, 0), (0, 0, 0))), (o, 1.0, _sweep((0, 0, 0), (0, 0, 0)))),
        ((o, r_touch, _sweep((0, 0, 0), (0, 0, 0))), (o, r_touch, _sweep((2, 0, 0), (2, 0, 0)))),
        ((o, 1.0, _sweep((0, 0, 0), (0, 0, 0))), (o, 1.0, _sweep((4, 0, 0), (4, 0, 0)))),
        ((o, 1.0, _sweep((-2, 0, 0), (0, 0, 0))), (o, 1.0, _sweep((2, 0, 0), (0, 0, 0)))),
        ((o, 1.0, _sweep((0, -20, 0), (0, 20, 0))), (o, 1.0, _sweep((0, 20, 0), (0, -20, 0)))),
        ((o, 1.0, _sweep((-3, 1, 0), (3, 1, 0))), (o, 1.0, _sweep((3, -1, 0), (-3, -1, 0)))),
    ]
    t, state, iters, _, _ = gpu.time_of_impact(pairs, **lim)
    names = [gpu.TOI_STATES[k] for k in state]
    assert names == ["overlapped", "touching", "separated", "touching", "touching", "separated"]
    assert list(iters) == [1, 1, 1, 2, 2, 7]
    assert t[0] == 0.0 and t[1] == 0.0 and t[2] == 1.0
    approx = ((F32(2) - F32(1)) + F32(lim["targetDepth"]) / F32(2)) / F32(2)
    assert abs(float(t[3]) - float(approx)) <= 1e-6
    assert abs(float(t[4]) - 0.4750375) <= 1e-6
    assert abs(float(t[5]) - 1.0) <= 1e-3
    # CollideEdgeCircleTouchingly (float build): 0.576901972
    conf = {"targetDepth": 0.0149999997, "tolerance": 0.0, "maxToiRootIters": 30, "maxToiIters": 20,
            "maxDistanceIters": 20}
    t, state, iters, _, _ = gpu.time_of_impact([(
        (((-40.0, 0.0), (40.0, 0.0)), 0.00999999977, _sweep((0, 0, 0), (0, 0, 0))),
        (o, 0.5, _sweep((-0.490861088, 0.49556452, 1.0125972), (-0.486600876, 0.494585991, 1.00495279))))],
        **conf)
    assert gpu.TOI_STATES[state[0]] == "touching" and iters[0] == 2
    assert abs(float(t[0]) - 0.576901972) <= 1e-6


def _random_shape(rng):
    k = int(rng.integers(0, 3))
    if k == 0:
        return ((0.0, 0.0),), float(F32(rng.uniform(0.1, 0.6)))
    if k == 1:
        a, b = rng.uniform(-1, 1, 2), rng.uniform(-1, 1, 2)
        return (tuple(a), tuple(b)), float(F32(0.01))
    n = int(rng.integers(3, 9))
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    r = rng.uniform(0.2, 0.8)
    hull = scenes.convex_hull([(r * np.cos(x), r * np.sin(x)) for x in ang])
    return tuple(map(tuple, hull)), float(F32(0.01))


@pytest.mark.parametrize("rotate", [False, True])
def test_toi_random_pairs_match_oracle(gpu_lib, rotate):
    rng = np.random.default_rng(41 if rotate else 40)
    pairs = []
    for _ in range(400):
        (va, ra), (vb, rb) = _random_shape(rng), _random_shape(rng)
        pa0 = rng.uniform(-3, 3, 2)
        pa1 = pa0 + rng.uniform(-4, 4, 2)
        pb0 = rng.uniform(-3, 3, 2)
        pb1 = pb0 + rng.uniform(-4, 4, 2)
        aa = rng.uniform(-3, 3, 2) if rotate else (0.0, 0.0)
        ab = rng.uniform(-3, 3, 2) if rotate else (0.0, 0.0)
        sa = np.asarray(_sweep((*pa0, aa[0]), (*pa1, aa[1]), 0.0, rng.uniform(-0.2, 0.2, 2) if rotate else (0, 0)),
                        F32)
        sb = np.asarray(_sweep((*pb0, ab[0]), (*pb1, ab[1])), F32)
        pairs.append(((va, ra, sa), (vb, rb, sb)))
    t, state, iters, dist_it, root_it = gpu.time_of_impact(pairs)
    ot, ostate = np.zeros(len(pairs), F32), []
    for i, ((va, ra, sa), (vb, rb, sb)) in enumerate(pairs):
        time, st, it, _, _ = oracle.time_of_impact(va, ra, sa[:7], sa[7:9], vb, rb, sb[:7], sb[7:9])
        ot[i] = time
        ostate.append(st)
    gstate = [gpu.TOI_STATES[k] for k in state]
    if not rotate:
        # no rotation: cos/sin of 0 are exact, so every operation matches the oracle
        assert gstate == ostate
        np.testing.assert_array_equal(t, ot)
    else:
        same = np.asarray([a == b for a, b in zip(gstate, ostate)])
        assert same.mean() >= 0.97, same.mean()
        np.testing.assert_allclose(t[same], ot[same], atol=1e-4)
    assert {"touching", "separated"} <= set(gstate)


def helloworld_scene():
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, -10.0)
    sb.box(g, 50.0, 10.0)
    b = sb.body(scenes.DYNAMIC, 0.0, 4.0, acc=(0.0, float(F32(-9.8)), 0.0))
    sb.disk(b, 1.0)
    return sb.build()


def fired_disk(rng):
    """A frictionless disk (a bullet half the time) fired down at a long ground edge
    fast enough to pass through it within one step."""
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(g, (-500.0, 0.0), (500.0, 0.0), friction=0.0)
    flags = scenes.BF_DEFAULT | (scenes.BF_BULLET if rng.uniform() < 0.5 else 0)
    vx, vy = rng.uniform(-40, 40), -rng.uniform(80, 200)
    b = sb.body(scenes.DYNAMIC, rng.uniform(-5, 5), rng.uniform(1.5, 6.0), v=(vx, vy, 0.0),
                acc=(0.0, -10.0, 0.0), flags=flags)
    sb.disk(b, float(rng.uniform(0.1, 0.5)), density=1.0, friction=0.0)
    return sb.build()


def test_helloworld_with_toi_bit_exact(gpu_lib):
    sc = helloworld_scene()
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    events = 0
    for _ in range(60):
        st = g.step(doToi=1)
        ow.step(doToi=1)
        events += st["toiContactsFound"]
        gb, ob = g.bodies(), ow.bodies()
        np.testing.assert_array_equal(gb["pos"], ob["pos"])
        np.testing.assert_array_equal(gb["vel"], ob["vel"])
    assert events >= 1


def test_fired_disks_bit_exact_and_no_tunnelling(gpu_lib):
    rng = np.random.default_rng(7)
    worlds = [fired_disk(rng) for _ in range(24)]
    g = GpuBatch(worlds)
    g_off = GpuBatch(worlds)
    ows = [oracle.OracleWorld(w) for w in worlds]
    found = 0
    for step in range(20):
        st = g.step(doToi=1)
        g_off.step(doToi=0)
        found += st["toiContactsFound"]
        stats = [ow.step(doToi=1) for ow in ows]
        gb = g.bodies()
        for i, ow in enumerate(ows):
            ob = ow.bodies()
            base = int(g.body_base[i])
            np.testing.assert_array_equal(gb["pos"][base:base + 2], ob["pos"], err_msg=f"world {i} step {step}")
            np.testing.assert_array_equal(gb["vel"][base:base + 2], ob["vel"], err_msg=f"world {i} step {step}")
        assert st["toiContactsFound"] == sum(s["toiContactsFound"] for s in stats)
        assert st["toiSumPosIters"] == sum(s["toiSumPosIters"] for s in stats)
        assert st["toiSumVelIters"] == sum(s["toiSumVelIters"] for s in stats)
    assert found >= len(worlds)
    disks = np.asarray(g.body_base[:len(worlds)]) + 1
    assert (g.bodies()["pos"][disks, 1] > 0.0).all()
    assert (g_off.bodies()["pos"][disks, 1] < 0.0).any()  # without TOI some pass through


def test_bullets_stay_in_the_box(gpu_lib):
    # Fast mixed shapes in a closed box: without the TOI phase nearly all pass
    # through the walls within 60 steps; with it almost none do, as in the
    # reference (its sub-step limit lets a few through: the oracle counts them).
    size = 12.0
    worlds = [scenes.bullets(30, np.random.default_rng(60 + i), size=size) for i in range(8)]
    g, g_off = GpuBatch(worlds), GpuBatch(worlds)
    ows = [oracle.OracleWorld(w) for w in worlds]
    found = 0
    for _ in range(60):
        found += g.step(doToi=1)["toiContactsFound"]
        g_off.step(doToi=0)
        for ow in ows:
            ow.step(doToi=1)
    dyn = np.concatenate([np.arange(1, w.n_bodies) + int(g.body_base[i]) for i, w in enumerate(worlds)])
    outside = lambda p: int((~((np.abs(p[:, 0]) < size) & (np.abs(p[:, 1]) < size))).sum())
    escaped = outside(g.bodies()["pos"][dyn])
    escaped_without = outside(g_off.bodies()["pos"][dyn])
    escaped_oracle = sum(outside(ow.bodies()["pos"][1:]) for ow in ows)
    assert escaped_without >= 150
    assert escaped <= 8 and abs(escaped - escaped_oracle) <= 6, (escaped, escaped_oracle)
    assert found > 500


def test_bullets_one_step_matches_oracle(gpu_lib):
    sc = scenes.bullets(40, np.random.default_rng(5))
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    for _ in range(3):
        st = g.step(doToi=1)
        ost = ow.step(doToi=1)
    gb, ob = g.bodies(), ow.bodies()
    np.testing.assert_allclose(gb["pos"], ob["pos"], atol=1e-4, rtol=1e-5)
    np.testing.assert_allclose(gb["vel"], ob["vel"], atol=1e-3, rtol=1e-4)
    assert st["toiContactsFound"] == ost["toiContactsFound"]


def test_batch_equals_single_worlds(gpu_lib):
    worlds = [scenes.bullets(25, np.random.default_rng(80 + i), size=10.0) for i in range(5)]
    g = GpuBatch(worlds)
    singles = [GpuBatch([w]) for w in worlds]
    for _ in range(30):
        g.step(doToi=1)
        for s in singles:
            s.step(doToi=1)
    gb = g.bodies()
    for i, s in enumerate(singles):
        base, n = int(g.body_base[i]), worlds[i].n_bodies
        np.testing.assert_array_equal(gb["pos"][base:base + n], s.bodies()["pos"])
        np.testing.assert_array_equal(gb["vel"][base:base + n], s.bodies()["vel"])


def test_sub_stepping_bit_exact(gpu_lib):
    """SetSubStepping: each world's time-of-impact phase stops after one event and
    its next step skips the regular phase (AabbTreeWorld.cpp:1819-1823,
    :2206-2209).  Fired disks, 24 worlds in one batch whose steps complete at
    different times: IsStepComplete and the states equal the oracle's (pinned to
    the reference with sub-stepping in test_oracle_vs_reference) bit for bit."""
    rng = np.random.default_rng(17)
    worlds = [fired_disk(rng) for _ in range(24)]
    g = GpuBatch(worlds)
    g.set_sub_stepping(True)
    ows = [oracle.OracleWorld(w) for w in worlds]
    for ow in ows:
        ow.set_sub_stepping(True)
    incomplete = 0
    for step in range(30):
        g.step(doToi=1)
        for ow in ows:
            ow.step(doToi=1)
        gb = g.bodies()
        for i, ow in enumerate(ows):
            assert g.step_complete(i) == ow.is_step_complete(), (i, step)
            incomplete += 0 if ow.is_step_complete() else 1
            base = int(g.body_base[i])
            np.testing.assert_array_equal(gb["pos"][base:base + 2], ow.bodies()["pos"], err_msg=f"world {i} step {step}")
            np.testing.assert_array_equal(gb["vel"][base:base + 2], ow.bodies()["vel"], err_msg=f"world {i} step {step}")
    assert incomplete > 0
