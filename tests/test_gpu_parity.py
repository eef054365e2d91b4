"""GPU world step against the CPU oracle (which is pinned to the reference).

Parity bars (from the world-step specification):
  (1) broadphase pair sets and contact-feature IDs match exactly;
  (2) manifold points/normals agree within 1e-5 relative in FP32, and so do
      post-step states when both sides solve to convergence (the GPU sweeps
      constraints in colour order, the reference in island order);
  (3) long runs are compared through drift / penetration / stability metrics.
Everything goes through the C ABI (libprgpu.so) via playrho_gb300.gpu.
"""
import numpy as np
import pytest

import parity_util as pu
from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch, default_conf

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def pair_set(c):
    return set(map(tuple, np.asarray(c["proxy"]).astype(np.int64).tolist()))


def by_pair(c):
    return {tuple(int(x) for x in c["proxy"][k]): k for k in range(len(c["proxy"]))}


def assert_contacts_match(gc, oc, atol_scale=1.0):
    assert pair_set(gc) == pair_set(oc)
    gi, oi = by_pair(gc), by_pair(oc)
    for key, k in oi.items():
        j = gi[key]
        assert int(gc["touching"][j]) == int(oc["touching"][k]), key
        n = int(oc["count"][k])
        assert int(gc["count"][j]) == n, key
        assert int(gc["type"][j]) == int(oc["type"][k]), key
        np.testing.assert_array_equal(gc["features"][j][:n], oc["features"][k][:n], err_msg=str(key))
        if n:
            scale = max(1.0, float(np.abs(oc["local_point"][k]).max()))
            np.testing.assert_allclose(gc["local_normal"][j], oc["local_normal"][k], atol=RTOL * atol_scale)
            np.testing.assert_allclose(gc["local_point"][j], oc["local_point"][k], atol=RTOL * scale * atol_scale)
            np.testing.assert_allclose(gc["points"][j][:n, :2], oc["points"][k][:n, :2], atol=RTOL * scale * atol_scale)


def rebased(scene, pos, vel):
    """The scene with body positions (of the centre of mass) and velocities replaced."""
    s = scenes.Scene(**{f: getattr(scene, f) for f in scene.__dataclass_fields__})
    s.body_pos = np.ascontiguousarray(pos, dtype=np.float32)
    s.body_vel = np.ascontiguousarray(vel, dtype=np.float32)
    return s


def test_first_contacts_pyramid(gpu_lib):
    sc = scenes.pyramid()
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    g.step(deltaTime=0.0)
    ow.step(deltaTime=0.0)
    assert_contacts_match(g.contacts(), ow.contacts())
    np.testing.assert_array_equal(g.proxies(), ow.proxies()["aabb"])


def test_free_fall_is_bit_exact(gpu_lib):
    sc = scenes.pyramid()
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    for _ in range(10):
        g.step()
        ow.step()
        gb, ob = g.bodies(), ow.bodies()
        np.testing.assert_array_equal(gb["pos"], ob["pos"])
        np.testing.assert_array_equal(gb["vel"], ob["vel"])
    assert_contacts_match(g.contacts(), ow.contacts())


def _contacts_from_identical_transforms(batch, worlds, indices, min_contacts=1):
    """Rebases worlds `indices` of a stepped batch onto fresh GPU and oracle worlds
    with identical transforms (the oracle takes the GPU's), runs one zero-length
    step on both (proxies, pair search and the first manifold update, as the
    reference's first Step does) and compares every world's contacts."""
    sample = pu.rebased_worlds(batch, worlds, indices)
    g2 = GpuBatch(sample)
    ows = pu.oracle_worlds_with_gpu_transforms(g2, sample)
    g2.step(deltaTime=0.0)
    for o in ows:
        o.step(deltaTime=0.0)
    per = pu.split_contacts(g2.contacts(), g2.shape_base)
    gc = g2.contacts()
    total = 0
    for k, o in enumerate(ows):
        pu.assert_world_contacts_match(gc, per[k], o.contacts(), what=f"world {indices[k]}")
        total += len(per[k])
    assert total >= min_contacts
    return total


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_pair_sets_random_piles(gpu_lib, seed):
    # A settled pile rebased onto fresh worlds with identical transforms, then a
    # zero-length step: pair sets and features exact, manifolds within 1e-5.
    rng = np.random.default_rng(seed)
    sc = scenes.pile(150, rng, width=6.0)
    g = GpuBatch([sc])
    g.step_n(240)
    _contacts_from_identical_transforms(g, [sc], [0], min_contacts=20)


def test_headline_batch_sample_matches_oracle(gpu_lib):
    """The benchmark's batch (4096 worlds, log-uniform 16..2048 bodies, pyramids
    and piles, seed 1) after its 240 settling steps: 64 of its worlds (every 64th,
    so small and large, pyramids and piles) rebased onto identical transforms give
    the oracle's pair sets, features and manifolds."""
    worlds = scenes.batched_worlds(4096, seed=1)
    g = GpuBatch(worlds)
    g.step_n(240)
    idx = list(range(0, 4096, 64))
    n = _contacts_from_identical_transforms(g, worlds, idx, min_contacts=5000)
    assert n >= 5000


def crop(scene, keep):
    """The bodies of `scene` with keep[body] true, with their shapes (no joints)."""
    keep = np.asarray(keep, bool)
    new_id = np.cumsum(keep) - 1
    sk = keep[scene.shape_body]
    sb = scenes.SceneBuilder()
    for b in np.flatnonzero(keep):
        sb.body(int(scene.body_type[b]), *(float(x) for x in scene.body_pos[b]), v=tuple(scene.body_vel[b]),
                acc=tuple(scene.body_acc[b]), damp=tuple(scene.body_damp[b]), flags=int(scene.body_flags[b]))
    for s in np.flatnonzero(sk):
        vo, nv = int(scene.shape_voff[s]), int(scene.shape_nv[s])
        sb._shape(int(new_id[scene.shape_body[s]]), int(scene.shape_kind[s]),
                  [tuple(v) for v in scene.verts[vo:vo + nv]], float(scene.shape_radius[s]),
                  float(scene.shape_density[s]), float(scene.shape_friction[s]),
                  float(scene.shape_restitution[s]), tuple(int(x) for x in scene.shape_filter[s]))
    return sb.build()


def test_large_world_crop_matches_oracle(gpu_lib):
    """The 100,000-shape box (1000 m, seed 0) after 60 steps, cropped to the
    bodies left of x = +100 m (60 % of the box: below the reference's 65,534-body
    limit) with the four walls, rebased onto identical transforms: pair sets,
    features and manifolds as the oracle's."""
    sc = scenes.large_box(100_000, 1000.0, seed=0)
    g = GpuBatch([sc])
    g.step_n(60)
    b = g.bodies()
    moved = pu.rebased(sc, b["pos"], b["vel"], b["local_center"])
    keep = (moved.body_type == scenes.STATIC) | (moved.body_pos[:, 0] < 100.0)
    cropped = crop(moved, keep)
    assert 50_000 < cropped.n_bodies <= 65_534
    g2 = GpuBatch([cropped])
    _contacts_from_identical_transforms(g2, [cropped], [0], min_contacts=500)


def test_chain_worlds_sample_matches_oracle(gpu_lib):
    """The chains workload's worlds (8,000 free disks and 3..8-gons plus 64 chains
    of 32 boxes on revolute joints, seed 3, dt 1/120, 10/4 iterations), the first
    two of its generator after its 120 settling steps, rebased onto identical
    transforms: pair sets, features and manifolds as the oracle's."""
    rng = np.random.default_rng(3)
    worlds = [scenes.chains_world(rng) for _ in range(2)]
    g = GpuBatch(worlds)
    g.step_n(120, default_conf(deltaTime=1.0 / 120.0, regVelocityIters=10, regPositionIters=4))
    _contacts_from_identical_transforms(g, worlds, [0, 1], min_contacts=3000)  # 4075 of them


def test_disabled_body_has_no_proxy(gpu_lib):
    """A body created disabled gets no proxies (AabbTreeWorld.cpp:1040): it has no
    contacts although it overlaps others, and queries do not find its shapes."""
    sb = scenes.SceneBuilder()
    gnd = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(gnd, (-10.0, 0.0), (10.0, 0.0))
    a = sb.body(scenes.DYNAMIC, 0.0, 0.49, acc=scenes.GRAVITY)
    sb.box(a, 0.5, 0.5, density=1.0)
    off = sb.body(scenes.DYNAMIC, 0.3, 0.9, acc=scenes.GRAVITY,
                  flags=scenes.BF_ALLOW_SLEEP | scenes.BF_AWAKE)  # not enabled
    sb.disk(off, 0.5, density=1.0)
    c = sb.body(scenes.DYNAMIC, 2.0, 0.45, acc=scenes.GRAVITY)
    sb.disk(c, 0.5, density=1.0)
    sc = sb.build()
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    assert len(g.query_aabb(0, (-20.0, -20.0, 20.0, 20.0))) == 0  # before the first step: no proxies
    for _ in range(3):
        g.step()
        ow.step()
    gc, oc = g.contacts(), ow.contacts()
    per = pu.split_contacts(gc, g.shape_base)
    pu.assert_world_contacts_match(gc, per[0], oc, what="disabled body")
    assert all(2 not in key for key in per[0])  # shape 2 belongs to the disabled body
    found = set(g.query_aabb(0, (-20.0, -20.0, 20.0, 20.0)).tolist())
    assert found == {0, 1, 3}
    np.testing.assert_array_equal(g.bodies()["pos"][off], ow.bodies()["pos"][off])


def test_pyramid_long_run_settles(gpu_lib):
    sc = scenes.pyramid()
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    g.step_n(600)
    for _ in range(600):
        ow.step()
    gb, ob = g.bodies(), ow.bodies()
    dyn = sc.body_type == scenes.DYNAMIC
    # Both come to rest with the pyramid standing.  With 8 velocity iterations the
    # Gauss-Seidel solve is far from converged, so the colour order and the
    # island order settle a few boxes at slightly different places: heights agree
    # within 2 cm (no box dropped), lateral positions within 10 cm.
    dx = np.abs(gb["pos"][dyn, 0] - ob["pos"][dyn, 0]).max()
    dy = np.abs(gb["pos"][dyn, 1] - ob["pos"][dyn, 1]).max()
    assert dy < 0.02, f"heights differ by {dy:.4f} m"
    assert dx < 0.10, f"lateral positions differ by {dx:.4f} m"
    assert int(gb["awake"].sum()) == int(ob["awake"].sum()) == 0, (int(gb["awake"].sum()), int(ob["awake"].sum()))


def test_batch_equals_single_worlds(gpu_lib):
    rng = np.random.default_rng(7)
    worlds = [scenes.pyramid(rows=5), scenes.pile(60, rng, width=5.0), scenes.pyramid(rows=8),
              scenes.pile(90, rng, width=6.0)]
    batch = GpuBatch(worlds)
    singles = [GpuBatch([w]) for w in worlds]
    for _ in range(60):
        batch.step()
        for s in singles:
            s.step()
    bb = batch.bodies()
    for i, s in enumerate(singles):
        lo, hi = batch.body_base[i], batch.body_base[i + 1]
        sb = s.bodies()
        np.testing.assert_array_equal(bb["pos"][lo:hi], sb["pos"])
        np.testing.assert_array_equal(bb["vel"][lo:hi], sb["vel"])


def test_sweep_modes_agree(gpu_lib):
    """One CTA per world and one cooperative grid over the batch run the same
    colours in the same order: results agree bit for bit, joints included."""
    rng = np.random.default_rng(11)
    worlds = []
    for i in range(72):
        k = i % 4
        if k == 0:
            worlds.append(scenes.pyramid(rows=4 + i % 5))
        elif k == 1:
            worlds.append(scenes.pile(30 + i, rng, width=4.0 + (i % 3)))
        elif k == 2:
            worlds.append(scenes.chains_world(rng, n_free=12, n_chains=2, links=6))
        else:
            worlds.append(scenes.pile(8, rng, width=3.0))
    a = GpuBatch(worlds)  # per world; worlds of <= 256 bodies by a warp, the rest by a CTA
    b = GpuBatch(worlds)  # one cooperative grid
    c = GpuBatch(worlds)  # per world, every world by a whole CTA
    e = GpuBatch(worlds)  # per world, every world by a warp
    assert a.sweep_mode() == "per_world"  # 72 worlds: the default is per world
    assert a.warp_world_max_bodies() == 256
    b.set_sweep_mode("grid")
    assert b.sweep_mode() == "grid"
    c.set_warp_world_max_bodies(0)
    e.set_warp_world_max_bodies(2 ** 32 - 1)
    f = GpuBatch(worlds)  # per world, body state staged in shared memory
    f.set_stage_bytes(2048 * 44)
    assert f.stage_bytes() == 2048 * 44
    h = GpuBatch(worlds)  # per world, every world by a group of 64 threads
    h.set_warp_world_max_bodies(0)
    h.set_group_world_max_bodies(1024)
    assert h.group_world_max_bodies() == 1024
    k = GpuBatch(worlds)  # warps up to 32 bodies, groups up to 64, CTAs above; staged
    k.set_warp_world_max_bodies(32)
    k.set_group_world_max_bodies(64)
    k.set_stage_bytes(2048 * 44)
    for i in range(90):
        for g in (a, b, c, e, f, h, k):
            g.step()
        if i == 40:  # switching schedule mid-run recaptures the step and changes nothing
            a.set_warp_world_max_bodies(64)
            e.set_stage_bytes(1024 * 44)
            h.set_group_world_max_bodies(0)
            a.set_group_world_max_bodies(256)
    ba = a.bodies()
    for g in (b, c, e, f, h, k):
        bg = g.bodies()
        np.testing.assert_array_equal(ba["pos"], bg["pos"])
        np.testing.assert_array_equal(ba["vel"], bg["vel"])
        assert pair_set(a.contacts()) == pair_set(g.contacts())


def test_autotune_keeps_results(gpu_lib):
    """The autotuner times schedules on the live batch; the batch ends where
    plain steps would have taken it."""
    rng = np.random.default_rng(5)
    worlds = [scenes.pile(20 + 7 * i, rng, width=4.0) for i in range(80)]
    a, b = GpuBatch(worlds), GpuBatch(worlds)
    best = a.autotune(steps_per_candidate=2)
    assert best["sweeps"] in ("grid", "per_world") and best["step_ms"] > 0
    assert best["group_world_max_bodies"] in (0, 256, 512, 1024)
    # the grid, 3 staging sizes x 5 warp-world limits, 2 x 3 group limits; the 3 fastest again
    n_cand = 1 + 3 * 5 + 2 * 3 + 3
    b.step_n(n_cand * 3)
    np.testing.assert_array_equal(a.bodies()["pos"], b.bodies()["pos"])
    np.testing.assert_array_equal(a.bodies()["vel"], b.bodies()["vel"])


def test_deterministic(gpu_lib):
    rng = np.random.default_rng(11)
    sc = scenes.pile(200, rng, width=6.0)
    a, b = GpuBatch([sc]), GpuBatch([sc])
    a.step_n(80)
    b.step_n(80)
    np.testing.assert_array_equal(a.bodies()["pos"], b.bodies()["pos"])


def _stack(n=3, gap=0.0175):
    # Boxes resting with their skins overlapping by 2.5 mm (inside the 5 mm linear
    # slop), so the position solver, whose fixed point is order dependent, makes
    # no correction and the step is decided by the velocity solve alone.
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(g, (-5.0, 0.0), (5.0, 0.0), friction=0.6)
    for i in range(n):
        b = sb.body(scenes.DYNAMIC, 0.1 * i, 0.5 + gap + (1.0 + gap) * i, acc=scenes.GRAVITY)
        sb.box(b, 0.5, 0.5, density=1.0, friction=0.6)
    return sb.build()


def test_one_step_at_convergence(gpu_lib):
    # Resting stack, both sides iterated far past convergence: post-step
    # velocities and positions agree within 1e-5 relative.
    sc = _stack(3)
    conf = dict(regVelocityIters=400, regPositionIters=30, regMinSeparation=float("inf"))
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    for _ in range(3):
        g.step(**conf)
        ow.step(**conf)
    gb, ob = g.bodies(), ow.bodies()
    dp = np.abs(gb["pos"] - ob["pos"]) / np.maximum(1.0, np.abs(ob["pos"]))
    dv = np.abs(gb["vel"] - ob["vel"]) / np.maximum(1.0, np.abs(ob["vel"]))
    assert dp.max() <= 1e-5, f"relative position difference {dp.max():.3g}"
    assert dv.max() <= 1e-5, f"relative velocity difference {dv.max():.3g}"


def test_revolute_chain(gpu_lib):
    rng = np.random.default_rng(3)
    sc = scenes.chains_world(rng, n_free=40, n_chains=3, links=6)
    g, ow = GpuBatch([sc]), oracle.OracleWorld(sc)
    for _ in range(30):
        g.step()
        ow.step()
    gb, ob = g.bodies(), ow.bodies()
    # chains hang from static anchors; link positions agree closely
    d = np.abs(gb["pos"] - ob["pos"]).max()
    assert d < 5e-3, f"positions differ by {d:.4g}"
