"""Failure paths without a GPU fault: a step that runs out of contact capacity
(with capacity growth: undone, capacities doubled, run again; without: the
PRGPU_ECAPACITY status), and a bounded grid-barrier wait made to give up at once
through the host-set wait limit (PRGPU_ETIMEOUT, the context stays usable)."""
import numpy as np
import pytest

from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch, PrgpuError

pytestmark = pytest.mark.gpu


def _pile():
    return scenes.pile(300, np.random.default_rng(5))


def test_capacity_growth_reruns_the_step(gpu_lib):
    big = GpuBatch([_pile()])
    small = GpuBatch([_pile()], contact_capacity=48, candidate_capacity=48)
    small.set_capacity_growth(True)
    for _ in range(120):
        big.step()
        small.step()
    c, k = small.capacities()
    assert c > 48 and k > 48  # the capacities grew
    assert small.contact_count() > 48
    # the same run as with the larger capacities from the start, bit for bit
    np.testing.assert_array_equal(small.bodies()["pos"], big.bodies()["pos"])
    np.testing.assert_array_equal(small.bodies()["vel"], big.bodies()["vel"])
    # step_n grows too
    small.step_n(30)
    big.step_n(30)
    np.testing.assert_array_equal(small.bodies()["pos"], big.bodies()["pos"])


def test_capacity_overflow_without_growth_reports_ecapacity(gpu_lib):
    g = GpuBatch([_pile()], contact_capacity=48, candidate_capacity=48)
    with pytest.raises(PrgpuError) as e:
        for _ in range(120):
            g.step()
    assert e.value.code == 3  # PRGPU_ECAPACITY


def test_barrier_wait_limit_gives_up(gpu_lib):
    worlds = [scenes.pile(200, np.random.default_rng(6 + k)) for k in range(4)]
    g = GpuBatch(worlds)
    g.set_sweep_mode("grid")  # one cooperative launch with a grid barrier per colour
    g.step_n(40)  # contacts to solve
    g.set_wait_limit(1)  # the first wait gives up
    with pytest.raises(PrgpuError) as e:
        g.step()
    assert e.value.code == 4  # PRGPU_ETIMEOUT
    # the context stays usable: a fresh batch steps and matches a reference run
    a, b = GpuBatch(worlds), GpuBatch(worlds)
    a.step_n(10)
    b.step_n(10)
    np.testing.assert_array_equal(a.bodies()["pos"], b.bodies()["pos"])
