"""Spatial queries on the GPU over the step's LBVH: Query (DynamicTree.cpp:673-710)
and RayCast (RayCastOutput.cpp:41-337), against the oracle's restatement (pinned
bit for bit to the reference in test_oracle_vs_reference) with identical body
transformations on both sides, and against a brute-force scan of the GPU's own
fat AABBs for the tree walk."""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch

pytestmark = pytest.mark.gpu


def _rays(rng, n, half):
    a = np.stack([rng.uniform(-half, half, n), rng.uniform(0.0, 5.0, n)], 1)
    b = np.stack([rng.uniform(-half, half, n), rng.uniform(-1.0, 5.0, n)], 1)
    b[: n // 8, 0] = a[: n // 8, 0]
    b[n // 8: n // 4] = a[n // 8: n // 4] + rng.uniform(-0.5, 0.5, (n // 4 - n // 8, 2))
    f = rng.uniform(0.2, 1.0, n)
    f[::3] = 1.0
    return np.concatenate([a, b, f[:, None]], 1).astype(np.float32)


def _settled(seed, n=150, steps=120):
    sc = scenes.pile(n, np.random.default_rng(seed))
    g = GpuBatch([sc])
    g.step_n(steps)
    o = oracle.OracleWorld(sc)
    o.step(deltaTime=0.0)  # creates the proxies
    o.set_body_xf(g.bodies()["xf"])  # the GPU's transformations, bit for bit
    return sc, g, o


@pytest.mark.parametrize("seed", [48, 50])
def test_raycast_all_and_nearest_match_oracle(gpu_lib, seed):
    sc, g, o = _settled(seed)
    rays = _rays(np.random.default_rng(seed + 1), 300, 18.0)
    hits = 0
    shapes, near = g.raycast(np.zeros(len(rays), np.uint32), rays)
    for k, r in enumerate(rays):
        want = o.raycast(r[0:2], r[2:4], r[4])
        got = g.raycast_all(0, r)
        assert len(got) == len(want), (k, got, want)
        for a, b in zip(got, want):
            assert a[0] == b[0] and np.array_equal(np.float32(a[1:]), np.float32(b[1:])), (k, a, b)
        hits += len(got)
        # the nearest hit (ClipRay): least fraction, ties to the lower shape
        if want:
            best = min(want, key=lambda h: (h[1], h[0]))
            assert shapes[k] == best[0] and np.array_equal(near[k], np.float32(best[1:])), (k, shapes[k], best)
        else:
            assert shapes[k] == -1
    assert hits > 100


def test_query_walks_the_tree(gpu_lib):
    worlds = [scenes.pile(200, np.random.default_rng(60 + k)) for k in range(3)]
    g = GpuBatch(worlds)
    g.step_n(60)
    boxes_all = g.proxies()
    rng = np.random.default_rng(7)
    n = 3000
    wq = rng.integers(0, 3, n).astype(np.uint32)
    c = np.stack([rng.uniform(-25, 25, n), rng.uniform(-1, 30, n)], 1)
    e = rng.uniform(0.05, 6.0, (n, 2))
    boxes = np.concatenate([c - e, c + e], 1).astype(np.float32)
    counts, found = g.query_aabbs(wq, boxes, capacity=512)
    total = 0
    for k in range(n):
        lo, hi = int(g.shape_base[wq[k]]), int(g.shape_base[wq[k] + 1])
        a = boxes_all[lo:hi]
        q = boxes[k]
        hit = (np.maximum(a[:, 0], q[0]) <= np.minimum(a[:, 2], q[2])) & \
              (np.maximum(a[:, 1], q[1]) <= np.minimum(a[:, 3], q[3]))
        want = np.flatnonzero(hit)
        assert counts[k] == len(want) and np.array_equal(found[k], want), k
        total += len(want)
        if k < 50:  # the single-query entry point agrees
            assert np.array_equal(g.query_aabb(int(wq[k]), q), want)
    assert total > 1000


def test_queries_before_the_first_step_find_nothing(gpu_lib):
    g = GpuBatch([scenes.pile(20, np.random.default_rng(1))])
    counts, _ = g.query_aabbs([0], [[-100, -100, 100, 100]])
    assert counts[0] == 0
    shapes, _ = g.raycast([0], [[-50, 1, 50, 1, 1]])
    assert shapes[0] == -1
