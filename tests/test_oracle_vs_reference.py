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
