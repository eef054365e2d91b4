"""prgpu_query_aabb (Query over a world's broadphase tree) against the oracle's
fat AABBs: frictionless disks step bit for bit like the oracle, so the proxies'
fat AABBs agree and every query must return the same shapes."""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300.gpu import GpuBatch

from test_gpu_events import bouncing_disks

pytestmark = pytest.mark.gpu


def overlapping(aabbs, q):
    """TestOverlap(leaf, query) as the reference evaluates it, per axis."""
    lo = np.maximum(aabbs[:, 0:2], q[0:2])
    hi = np.minimum(aabbs[:, 2:4], q[2:4])
    return np.nonzero(np.all(hi >= lo, axis=1))[0]


def test_query_matches_oracle(gpu_lib):
    worlds = [bouncing_disks(np.random.default_rng(80 + k)) for k in range(3)]
    g = GpuBatch(worlds)
    ows = [oracle.OracleWorld(w) for w in worlds]
    rng = np.random.default_rng(5)
    for step in range(30):
        g.step()
        for ow in ows:
            ow.step()
        if step % 10 != 9:
            continue
        for i, ow in enumerate(ows):
            px = ow.proxies()
            shape_of = px["bsc"][:, 1]
            aabbs = px["aabb"].astype(np.float32)
            for _ in range(20):
                c = rng.uniform([-24.0, -1.0], [24.0, 4.0])
                h = rng.uniform(0.1, 6.0, 2)
                q = np.array([c[0] - h[0], c[1] - h[1], c[0] + h[0], c[1] + h[1]], np.float32)
                want = np.sort(shape_of[overlapping(aabbs, q)])
                np.testing.assert_array_equal(g.query_aabb(i, q), want)
            everything = np.array([-1e6, -1e6, 1e6, 1e6], np.float32)
            assert len(g.query_aabb(i, everything)) == worlds[i].n_shapes
            assert len(g.query_aabb(i, np.array([500.0, 500.0, 501.0, 501.0], np.float32))) == 0
