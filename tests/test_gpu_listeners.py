"""PreSolveContact / PostSolveContact on the GPU: the solve records of each step
(prgpu_download_solve_records) against the oracle's listener calls, which
tests/test_oracle_vs_reference.py pins call for call to the reference.

The oracle replays the GPU's sweep order (prgpu_download_sweep_order) so that
both solve the same Gauss-Seidel sequence; contacts are named by their shapes."""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch

pytestmark = pytest.mark.gpu


def _by_shapes(g):
    c = g.contacts()
    return {int(s): (int(min(p)), int(max(p)), int(t))
            for s, p, t in zip(g.contact_slots(), c["proxy"], c["touching"])}


def _compare(scene, steps):
    g, o = GpuBatch([scene]), oracle.OracleWorld(scene)
    g.set_solve_records(True)
    n_pre = n_post = 0
    for step in range(steps):
        g.step()
        o.set_solve_order(g.sweep_order())
        o.step()
        calls = o.solve_calls()
        rec = g.solve_records()
        shapes = _by_shapes(g)
        post_o = {(c[1], c[2]): c for c in calls if c[0] == 4}
        pre_o = {(c[1], c[2]) for c in calls if c[0] == 3}
        post_g, pre_g = {}, set()
        for k in range(len(rec["slot"])):
            lo, hi, touching = shapes[int(rec["slot"][k])]
            if rec["solved"][k]:
                post_g[(lo, hi)] = k
            if rec["phases"][k] and touching:
                pre_g.add((lo, hi))
        # PostSolveContact: the same contacts, point counts and iteration
        # arguments; impulses as the solve's (same order, same arithmetic)
        assert set(post_g) == set(post_o), step
        for key, k in post_g.items():
            c = post_o[key]
            assert (int(rec["count"][k]), int(rec["iter"][k])) == (c[3], c[4]), (step, key)
            np.testing.assert_allclose(rec["imp"][k], c[5:9], rtol=1e-4, atol=1e-5, err_msg=f"step {step} {key}")
        # PreSolveContact: every updated contact that touches afterwards
        assert pre_g == pre_o, step
        n_pre += len(pre_g)
        n_post += len(post_g)
    return n_pre, n_post


def test_solve_records_pyramid(gpu_lib):
    n_pre, n_post = _compare(scenes.pyramid(rows=8), 30)
    assert n_pre > 300 and n_post > 300


@pytest.mark.parametrize("seed", [44, 45])
def test_solve_records_piles(gpu_lib, seed):
    n_pre, n_post = _compare(scenes.pile(150, np.random.default_rng(seed)), 40)
    assert n_pre > 40 and n_post > 40


def test_solve_records_off_by_default(gpu_lib):
    g = GpuBatch([scenes.pyramid(rows=4)])
    g.step_n(30)  # the boxes have landed on each other
    rec = g.solve_records()
    assert len(rec["slot"]) > 0 and not rec["solved"].any()  # updates are still reported
    g.set_solve_records(True)
    g.step()
    assert g.solve_records()["solved"].any()
    g.set_solve_records(False)
    g.step()
    assert not g.solve_records()["solved"].any()
