"""Sensor contacts on the GPU: touching by TestOverlap (GJK distance of the two
shapes against their total vertex radius, Distance.cpp:205-216, called by
Update at AabbTreeWorld.cpp:2620-2634), no manifold, BeginContact / EndContact
for them; against the oracle, which test_oracle_vs_reference pins to the
reference on the same scene kind."""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import ContactEvents, GpuBatch

pytestmark = pytest.mark.gpu


def _sensor_touching(pairs, touching, sensors):
    return {(int(min(p)), int(max(p))) for p, t in zip(pairs, touching)
            if t and (int(p[0]) in sensors or int(p[1]) in sensors)}


def test_sensor_touching_and_events_match_oracle(gpu_lib):
    sc = scenes.sensor_scene(np.random.default_rng(47))
    sensors = set(np.flatnonzero(sc.shape_filter[:, 3]).tolist())
    g, o = GpuBatch([sc]), oracle.OracleWorld(sc)
    tracker = ContactEvents(g)
    seen = events = 0
    for step in range(150):
        got = tracker.step()[0]
        o.set_solve_order(g.sweep_order())
        o.step()
        assert got == o.events(), step
        gc, oc = g.contacts(), o.contacts()
        opairs = np.stack([oc["bsc_a"][:, 1], oc["bsc_b"][:, 1]], 1)
        tg = _sensor_touching(gc["proxy"], gc["touching"], sensors)
        assert tg == _sensor_touching(opairs, oc["touching"], sensors), step
        # sensors make no manifold
        sensor_rows = [k for k, p in enumerate(gc["proxy"]) if int(p[0]) in sensors or int(p[1]) in sensors]
        assert all(int(gc["count"][k]) == 0 for k in sensor_rows)
        seen += len(tg)
        events += sum(1 for e in got if e[1] in sensors or e[2] in sensors)
    assert seen > 50 and events > 10
