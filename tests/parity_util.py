"""Helpers shared by the GPU parity tests: rebasing scenes onto a batch's state,
giving the oracle the GPU's own transforms, and comparing contacts by shape."""
from __future__ import annotations

import numpy as np

from oracle import oracle
from playrho_gb300 import scenes

RTOL = 1e-5


def rebased(scene, pos_com, vel, lc):
    """The scene with each body moved to a centre-of-mass position pos_com (x y
    angle) and velocity (scenes.rebase)."""
    return scenes.rebase(scene, pos_com, vel, lc)


def rebased_worlds(batch, scenes_, indices):
    """Rebased copies of the batch's worlds `indices` at the batch's current state."""
    b = batch.bodies()
    out = []
    for k in indices:
        lo, hi = int(batch.body_base[k]), int(batch.body_base[k + 1])
        out.append(rebased(scenes_[k], b["pos"][lo:hi], b["vel"][lo:hi], b["local_center"][lo:hi]))
    return out


def oracle_worlds_with_gpu_transforms(batch, worlds, double=False):
    """One oracle world per scene, each given the transforms (p, cos, sin) the GPU
    batch computed for its bodies, so both sides start from identical transforms
    (CUDA's and the C library's sin/cos can round differently)."""
    xf = batch.bodies()["xf"]
    out = []
    for k, sc in enumerate(worlds):
        o = oracle.OracleWorld(sc, double=double)
        lo, hi = int(batch.body_base[k]), int(batch.body_base[k + 1])
        o.set_body_xf(xf[lo:hi])
        out.append(o)
    return out


def split_contacts(c, shape_base, body_base=None):
    """Splits a batch's contacts() into one dict per world with world-local shape IDs
    (and body IDs when body_base is given), keyed by the sorted shape pair."""
    sb = np.asarray(shape_base, dtype=np.int64)
    world = np.searchsorted(sb, c["proxy"][:, 0], side="right") - 1
    per = [dict() for _ in range(len(sb) - 1)]
    for i in range(len(world)):
        w = int(world[i])
        a, b = (int(x) - int(sb[w]) for x in c["proxy"][i])
        per[w][(min(a, b), max(a, b))] = i
    return per


def oracle_by_shape(oc):
    """The oracle's contacts keyed by the sorted shape pair (proxy numbers differ from
    shape IDs when some shapes have no proxy)."""
    out = {}
    for k in range(len(oc["count"])):
        a, b = int(oc["bsc_a"][k][1]), int(oc["bsc_b"][k][1])
        out[(min(a, b), max(a, b))] = k
    return out


def assert_world_contacts_match(gc, gidx, oc, what=""):
    """Pair set equal, touching / manifold type / point count / contact features exact,
    local normal, local point and manifold points within RTOL (absolute, scaled by the
    larger of 1 and the local point's magnitude)."""
    oidx = oracle_by_shape(oc)
    assert set(gidx) == set(oidx), f"{what}: pair sets differ by {len(set(gidx) ^ set(oidx))}"
    worst = 0.0
    for key, k in oidx.items():
        j = gidx[key]
        assert int(gc["touching"][j]) == int(oc["touching"][k]), (what, key)
        n = int(oc["count"][k])
        assert int(gc["count"][j]) == n, (what, key)
        assert int(gc["type"][j]) == int(oc["type"][k]), (what, key)
        np.testing.assert_array_equal(gc["features"][j][:n], oc["features"][k][:n], err_msg=f"{what} {key}")
        if n:
            scale = max(1.0, float(np.abs(oc["local_point"][k]).max()))
            d = max(float(np.abs(gc["local_normal"][j] - oc["local_normal"][k]).max()),
                    float(np.abs(gc["local_point"][j] - oc["local_point"][k]).max()) / scale,
                    float(np.abs(gc["points"][j][:n, :2] - oc["points"][k][:n, :2]).max()) / scale)
            worst = max(worst, d)
    assert worst <= RTOL, f"{what}: manifold differs by {worst:.3g} (relative)"
    return worst


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float((np.abs(a - b) / np.maximum(1.0, np.abs(b))).max()) if a.size else 0.0
