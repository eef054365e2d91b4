"""BeginContact / EndContact listener calls replayed from the GPU batch
(gpu.ContactEvents, over prgpu_download_contacts and prgpu_download_contact_seq)
against the oracle's, which are pinned to the reference's listener calls
(tests/test_oracle_vs_reference.py).

Bouncing frictionless disks never rotate and each touches only the ground, so the
GPU steps them bit for bit like the oracle and every touching change happens at
the same step: the replayed calls must equal the oracle's, in order."""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import ContactEvents, GpuBatch

pytestmark = pytest.mark.gpu


def bouncing_disks(rng, n=12):
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(g, (-2.0 * n, 0.0), (2.0 * n, 0.0), friction=0.0, restitution=0.6)
    for k in range(n):
        b = sb.body(scenes.DYNAMIC, -2.0 * n + 2.0 + 3.0 * k, float(rng.uniform(0.6, 3.0)),
                    v=(0.0, float(rng.uniform(-4.0, 2.0)), 0.0), acc=scenes.GRAVITY)
        sb.disk(b, float(rng.uniform(0.2, 0.5)), density=1.0, friction=0.0, restitution=0.6)
    return sb.build()


def test_replayed_events_equal_oracle(gpu_lib):
    worlds = [bouncing_disks(np.random.default_rng(60 + k)) for k in range(4)]
    g = GpuBatch(worlds)
    tracker = ContactEvents(g)
    ows = [oracle.OracleWorld(w) for w in worlds]
    counts = [0, 0]
    for step in range(120):
        got = tracker.step()
        for i, ow in enumerate(ows):
            ow.step()
            want = ow.events()
            assert got[i] == want, f"world {i} step {step}"
            counts[0] += sum(1 for e in want if e[0] == 1)
            counts[1] += sum(1 for e in want if e[0] == 2)
    assert counts[0] > 20 and counts[1] > 20  # the disks bounce: many begins and ends
