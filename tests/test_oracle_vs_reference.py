"""The CPU oracle against the PlayRho reference compiled from source, on scenes
not in the committed fixtures.  Skipped where the reference sources are absent."""
import numpy as np
import pytest

from oracle import oracle, refdriver
from playrho_gb300 import scenes

pytestmark = pytest.mark.skipif(not refdriver.available(), reason="reference sources not present")


def _compare(scene, steps, double=False, **conf):
    dumps = refdriver.run(scenes.scene_text(scene, conf), steps, double=double)
    ow = oracle.OracleWorld(scene, double=double)
    for n, d in zip(steps, dumps):
        for _ in range(n):
            st = ow.step(**conf)
        if conf.get("doToi"):
            assert [st[k] for k in oracle.TOI_STATS_INT_FIELDS] == d["toistats"][:14]
        b = ow.bodies()
        np.testing.assert_array_equal(b["pos"], d["bodies"]["pos"])
        np.testing.assert_array_equal(b["vel"], d["bodies"]["vel"])
        c = ow.contacts()
        np.testing.assert_array_equal(c["proxy"], d["contacts"]["proxy"])
        np.testing.assert_array_equal(c["count"], d["contacts"]["count"])
        np.testing.assert_array_equal(c["touching"], d["contacts"]["touching"])
        for k in range(len(c["count"])):
            m = int(c["count"][k])
            np.testing.assert_array_equal(c["features"][k][:m], d["contacts"]["features"][k][:m])


@pytest.mark.parametrize("seed", [11, 12])
def test_piles(seed):
    _compare(scenes.pile(250, np.random.default_rng(seed)), [1, 60, 120])


def test_small_pyramid_f64():
    _compare(scenes.pyramid(rows=8), [1, 100, 200], double=True)


def test_spinning_box():
    _compare(scenes.large_box(800, size=40.0, seed=4), [1, 40])


def test_chains():
    _compare(scenes.chains_world(np.random.default_rng(9), n_free=60, n_chains=3, links=6), [1, 80])


def test_disabled_bodies_have_no_proxies():
    # every fifth body of a pile is created disabled: the reference gives its shapes
    # no proxies (AabbTreeWorld.cpp:1040), so the proxy ranks, the contacts and the
    # steps follow without them
    sc = scenes.pile(120, np.random.default_rng(13))
    sc.body_flags[1::5] &= ~np.uint32(scenes.BF_ENABLED)
    _compare(sc, [1, 40, 90])


@pytest.mark.parametrize("seed", [21, 22])
def test_toi_bullets(seed):
    _compare(scenes.bullets(50, np.random.default_rng(seed)), [1, 20, 60], doToi=1)


def test_toi_pile_f64():
    _compare(scenes.pile(120, np.random.default_rng(23)), [1, 100, 150], double=True, doToi=1)


@pytest.mark.parametrize("kind", [1, 2, 3, 4, 5, 6, 7, 8, 9])
def test_joint_kinds(kind):
    # distance, rope, weld, friction, motor, prismatic, wheel, pulley and target joints
    # (stiff and soft, limits and motors on and off), with contacts
    _compare(scenes.joint_zoo(np.random.default_rng(30 + kind), per_kind=4, kinds=[kind], n_disks=6), [1, 30, 120])


def test_joint_zoo_f64():
    _compare(scenes.joint_zoo(np.random.default_rng(36)), [1, 80], double=True)


def _compare_events(scene, steps, double=False, **conf):
    """The oracle's BeginContact / EndContact calls equal the reference listeners'."""
    dumps = refdriver.run(scenes.scene_text(scene, conf), steps, double=double)
    ow = oracle.OracleWorld(scene, double=double)
    total = 0
    for n, d in zip(steps, dumps):
        evs = []
        for _ in range(n):
            ow.step(**conf)
            evs += ow.events()
        assert evs == d["events"]
        total += len(evs)
    return total


@pytest.mark.parametrize("seed", [41, 42])
def test_contact_events_piles(seed):
    assert _compare_events(scenes.pile(150, np.random.default_rng(seed)), [1, 40, 100]) > 0


def test_contact_events_bullets_with_toi():
    assert _compare_events(scenes.bullets(40, np.random.default_rng(43)), [1, 20, 40], doToi=1) > 0



@pytest.mark.parametrize("double", [False, True])
def test_gear_joints(double):
    # gear trains (revolute-revolute, one on a motor) and rack-and-pinion gears
    # (revolute-prismatic) with disks falling on them
    _compare(scenes.gear_scene(np.random.default_rng(61)), [1, 60, 120], double=double)


def _compare_solve_calls(scene, steps, double=False, **conf):
    """The oracle's PreSolveContact / PostSolveContact calls (contact, point count,
    iteration argument, impulses) equal the reference listeners', call for call."""
    dumps = refdriver.run(scenes.scene_text(scene, conf), steps, double=double)
    ow = oracle.OracleWorld(scene, double=double)
    kinds = {3: 0, 4: 0}
    for n, d in zip(steps, dumps):
        calls = []
        for _ in range(n):
            ow.step(**conf)
            calls += ow.solve_calls()
        assert calls == d["solve_calls"]
        for c in calls:
            kinds[c[0]] += 1
    return kinds


@pytest.mark.parametrize("seed", [44, 45])
def test_presolve_postsolve_piles(seed):
    kinds = _compare_solve_calls(scenes.pile(150, np.random.default_rng(seed)), [1, 40, 100])
    assert kinds[3] > 0 and kinds[4] > 0


def test_presolve_postsolve_with_toi_f64():
    # bullets: the time-of-impact islands report too (AabbTreeWorld.cpp:2053)
    kinds = _compare_solve_calls(scenes.bullets(40, np.random.default_rng(46)), [1, 20, 40], double=True, doToi=1)
    assert kinds[3] > 0 and kinds[4] > 0


@pytest.mark.parametrize("double", [False, True])
def test_sensors(double):
    # sensor zones and sensor bodies: touching by TestOverlap (AabbTreeWorld.cpp:
    # 2620-2634), no manifolds, Begin/EndContact for them
    sc = scenes.sensor_scene(np.random.default_rng(47))
    _compare(sc, [1, 60, 150], double=double)
    assert _compare_events(sc, [1, 60, 150], double=double) > 0
    dumps = refdriver.run(scenes.scene_text(sc, {}), [150], double=double)
    sensor_shapes = set(np.flatnonzero(sc.shape_filter[:, 3]).tolist())
    ev = [e for e in dumps[0]["events"] if e[1] in sensor_shapes or e[2] in sensor_shapes]
    assert len(ev) > 0  # sensors did begin or end touching


def _rays(rng, n, half):
    """Rays across a world of half-width `half`: random ends, a few vertical ones
    and short ones, maxFraction in (0, 1]."""
    a = np.stack([rng.uniform(-half, half, n), rng.uniform(0.0, 5.0, n)], 1)
    b = np.stack([rng.uniform(-half, half, n), rng.uniform(-1.0, 5.0, n)], 1)
    b[: n // 8, 0] = a[: n // 8, 0]  # vertical
    b[n // 8: n // 4] = a[n // 8: n // 4] + rng.uniform(-0.5, 0.5, (n // 4 - n // 8, 2))  # short
    f = rng.uniform(0.2, 1.0, n)
    f[::3] = 1.0
    return np.concatenate([a, b, f[:, None]], 1)


@pytest.mark.parametrize("double", [False, True])
def test_raycast(double):
    # RayCast(World, RayCastInput, callback) (RayCastOutput.cpp:301-337) answering
    # ResetRay: every shape hit, its point and normal, after the pile has settled
    # into contact; the reference reports them in tree order, the oracle in shape order
    sc = scenes.pile(150, np.random.default_rng(48))
    rays = _rays(np.random.default_rng(49), 200, 18.0)
    ref = refdriver.run_rays(scenes.scene_text(sc, {}), 120, rays, double=double)
    ow = oracle.OracleWorld(sc, double=double)
    for _ in range(120):
        ow.step()
    hits = 0
    for r, want in zip(rays, ref):
        got = ow.raycast(r[0:2], r[2:4], r[4])
        assert [(g[0], g[2], g[3], g[4], g[5]) for g in got] == sorted(want), r
        hits += len(got)
    assert hits > 100


@pytest.mark.parametrize("double", [False, True])
def test_multi_child_shapes(double):
    # a ChainShapeConf terrain (one proxy per edge child) and bodies of MultiShapeConf
    # hulls: proxies, contact keys and features per child, mass data of the whole
    # shape (ChainShapeConf.cpp:113-147, MultiShapeConf.cpp:35-57), states
    _compare(scenes.multi_child_scene(np.random.default_rng(51)), [1, 60, 150], double=double)


@pytest.mark.parametrize("double", [False, True])
def test_toi_sub_stepping(double):
    # SetSubStepping: the time-of-impact phase stops after one event a step and the
    # next Step skips the regular phase until an event loop finds nothing
    # (AabbTreeWorld.cpp:1819-1823, :2206-2209)
    sc = scenes.bullets(40, np.random.default_rng(57))
    steps = [1, 1, 1, 5, 20, 40]
    dumps = refdriver.run("substep 1\n" + scenes.scene_text(sc, {"doToi": 1}), steps, double=double)
    ow = oracle.OracleWorld(sc, double=double)
    ow.set_sub_stepping(True)
    incomplete = 0
    for n, d in zip(steps, dumps):
        for _ in range(n):
            ow.step(doToi=1)
        assert int(ow.is_step_complete()) == d["complete"]
        incomplete += 1 - d["complete"]
        b = ow.bodies()
        np.testing.assert_array_equal(b["pos"], d["bodies"]["pos"])
        np.testing.assert_array_equal(b["vel"], d["bodies"]["vel"])
    assert incomplete > 0
