"""Multi-child shapes on the GPU: a ChainShapeConf terrain (each edge child its own
proxy and contacts) and bodies of MultiShapeConf hulls, against the oracle (pinned
bit for bit to the reference on the same scene kind in test_oracle_vs_reference)."""
import numpy as np
import pytest

import parity_util as pu
from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch

pytestmark = pytest.mark.gpu


def test_multi_child_contacts_from_identical_transforms(gpu_lib):
    # settled on the terrain, rebased onto identical transformations: pair sets and
    # features per child exact, manifolds within 1e-5
    worlds = [scenes.multi_child_scene(np.random.default_rng(52 + k)) for k in range(3)]
    g = GpuBatch(worlds)
    g.step_n(150)
    sample = pu.rebased_worlds(g, worlds, [0, 1, 2])
    g2 = GpuBatch(sample)
    ows = pu.oracle_worlds_with_gpu_transforms(g2, sample)
    g2.step(deltaTime=0.0)
    for o in ows:
        o.step(deltaTime=0.0)
    per = pu.split_contacts(g2.contacts(), g2.shape_base)
    gc = g2.contacts()
    total = 0
    for k, o in enumerate(ows):
        pu.assert_world_contacts_match(gc, per[k], o.contacts(), what=f"world {k}")
        total += len(per[k])
    assert total > 100


def test_multi_child_steps_match_oracle(gpu_lib):
    # the oracle replays the GPU's sweep order: one step from the start within 1e-5,
    # 60 steps within 1e-4
    sc = scenes.multi_child_scene(np.random.default_rng(55))
    g, o = GpuBatch([sc]), oracle.OracleWorld(sc)
    for step in range(60):
        g.step()
        o.set_solve_order(g.sweep_order())
        o.step()
        tol = 1e-5 if step == 0 else 1e-4
        if step in (0, 29, 59):
            np.testing.assert_allclose(g.bodies()["pos"], o.bodies()["pos"], rtol=tol, atol=tol, err_msg=f"step {step}")
            np.testing.assert_allclose(g.bodies()["vel"], o.bodies()["vel"], rtol=tol, atol=tol, err_msg=f"step {step}")
    assert int(g.contacts()["touching"].sum()) > 8
