"""Host-side batch preparation of the C ABI (mass data, centre positions) against
the oracle, which matches the reference bit for bit.  Runs without a GPU."""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import build, gpu, scenes


@pytest.fixture(scope="module")
def lib():
    build.build()
    return gpu.load_library()


def _cases():
    rng = np.random.default_rng(1)
    return {
        "pyramid": scenes.pyramid(),
        "pile": scenes.pile(120, rng),
        "box": scenes.large_box(400, size=40.0, seed=0),
        "chains": scenes.chains_world(np.random.default_rng(3), n_free=30, n_chains=2, links=5),
        "push": scenes.push_worlds(1)[0],
        # multi-child shapes: a chain terrain and bodies of MultiShapeConf hulls (one
        # Attach each, mass data of the whole shape)
        "multi": scenes.multi_child_scene(np.random.default_rng(5)),
    }


@pytest.mark.parametrize("name", list(_cases().keys()))
def test_prepare_matches_oracle(lib, name):
    sc = _cases()[name]
    hp = gpu.prepare_bodies([sc])
    ob = oracle.OracleWorld(sc).bodies()
    np.testing.assert_array_equal(hp["pos"], ob["pos"])
    np.testing.assert_array_equal(hp["vel"], ob["vel"])
    np.testing.assert_array_equal(hp["inv_mass"], ob["inv_mass"])
    np.testing.assert_array_equal(hp["inv_rot_inertia"], ob["inv_rot_inertia"])


def test_prepare_batch_is_concatenation(lib):
    c = _cases()
    worlds = [c["pyramid"], c["pile"], c["chains"]]
    whole = gpu.prepare_bodies(worlds)
    parts = [gpu.prepare_bodies([w]) for w in worlds]
    np.testing.assert_array_equal(whole["pos"], np.concatenate([p["pos"] for p in parts]))


def test_invalid_descriptions_rejected(lib):
    sc = scenes.pyramid(rows=2)
    bad = scenes.Scene(**{f: getattr(sc, f) for f in sc.__dataclass_fields__})
    bad.shape_nv = bad.shape_nv.copy()
    bad.shape_nv[0] = 1  # an edge with one vertex
    with pytest.raises(gpu.PrgpuError):
        gpu.prepare_bodies([bad])


def test_multi_child_owner_rules(lib):
    sc = scenes.multi_child_scene(np.random.default_rng(6))
    bad = scenes.Scene(**{f: getattr(sc, f) for f in sc.__dataclass_fields__})
    bad.shape_owner = bad.shape_owner.copy()
    k = int(np.flatnonzero(bad.shape_owner >= 0)[3])
    bad.shape_owner[k] = k + 5  # a child before its shape's first child
    with pytest.raises(gpu.PrgpuError):
        gpu.prepare_bodies([bad])


def test_library_exports(lib):
    import os
    import re
    header = os.path.join(os.path.dirname(__file__), "..", "include", "prgpu.h")
    declared = set(re.findall(r"^int (prgpu_\w+)\(", open(header).read(), re.M))
    assert declared >= set(gpu.exported_symbols())
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert lib.prgpu_abi_version() == 5


def test_convex_hull_matches_scene_builder(lib):
    import ctypes
    rng = np.random.default_rng(4)
    for _ in range(50):
        n = int(rng.integers(3, 9))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        r = rng.uniform(0.1, 0.6)
        pts = [(r * np.cos(a), r * np.sin(a)) for a in ang]
        want = scenes.convex_hull(pts)
        xy = np.asarray(pts, np.float32).reshape(-1)
        out = np.zeros_like(xy)
        m = lib.prgpu_convex_hull(xy.ctypes.data, n, ctypes.c_float(0.005), out.ctypes.data)
        np.testing.assert_array_equal(out[:2 * m].reshape(-1, 2), np.asarray(want, np.float32))
