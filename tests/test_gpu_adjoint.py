"""StepAdjoint: the reverse pass against the FP64 tangent (dot-product test),
against finite differences, and the differentiable restatement against the
forward kernels (replay, bit for bit).
"""
import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch, default_conf

pytestmark = pytest.mark.gpu


def dynamic_mask(batch_scenes):
    return np.concatenate([s.body_type == scenes.DYNAMIC for s in batch_scenes])


def test_dot_product_and_replay(gpu_lib):
    """<ybar, J xdot> (FP64 tangent) equals <J^T ybar, xdot> (adjoint) over a
    window of 12 steps with checkpoints every 4, on pushed boxes in contact."""
    worlds = scenes.push_worlds(6, seed=2)
    g = GpuBatch(worlds)
    conf = default_conf(minStillTimeToSleep=1e9)  # keep every body awake in the window
    g.step_n(40, conf)  # boxes land; the disk meets the first ones
    g.adjoint_begin(4)
    g.adjoint_forward(12, conf)
    info = g.adjoint_info()
    rng = np.random.default_rng(0)
    dyn = dynamic_mask(worlds)
    n, s = g.n_bodies, g.n_shapes
    ybar_p = rng.standard_normal((n, 3)) * dyn[:, None]
    ybar_v = rng.standard_normal((n, 3)) * dyn[:, None]
    xdot_p = rng.standard_normal((n, 3)) * dyn[:, None] * 1e-2
    xdot_v = rng.standard_normal((n, 3)) * dyn[:, None] * 1e-1
    xdot_f = rng.standard_normal(s) * 1e-2
    adj = g.adjoint_backward(ybar_p, ybar_v)
    tan = g.adjoint_tangent(xdot_p, xdot_v, xdot_f)
    info = g.adjoint_info()
    assert info["steps"] == 12
    assert info["replay_mismatches"] == 0, info
    assert info["tape_overflows"] == 0, info
    lhs = float((ybar_p * tan["pos"]).sum() + (ybar_v * tan["vel"]).sum())
    rhs = float((adj["pos"].astype(np.float64) * xdot_p).sum() + (adj["vel"].astype(np.float64) * xdot_v).sum() +
                (adj["friction"].astype(np.float64) * xdot_f).sum())
    scale = max(abs(lhs), abs(rhs), 1e-12)
    print(f"\ndot-product test: <ybar, J xdot> = {lhs:.9e}, <J^T ybar, xdot> = {rhs:.9e}, "
          f"rel diff {abs(lhs - rhs) / scale:.2e}")
    assert abs(lhs - rhs) <= 1e-4 * scale
    # the window leaves the batch where the forward steps left it
    b = g.bodies()
    g.adjoint_end()
    g2 = GpuBatch(worlds)
    g2.step_n(52, conf)
    np.testing.assert_array_equal(b["pos"], g2.bodies()["pos"])


def _fd_scene():
    """A disk pushing three boxes along the ground (no stacking)."""
    sb = scenes.SceneBuilder()
    gnd = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(gnd, (-20.0, 0.0), (40.0, 0.0), friction=0.5)
    d = sb.body(scenes.DYNAMIC, 0.0, 0.5, v=(6.0, 0.0, 0.0), acc=scenes.GRAVITY)
    sb.disk(d, 0.5, density=1.0, friction=0.5)
    for x in (2.0, 3.2, 4.4):
        b = sb.body(scenes.DYNAMIC, x, 0.5, acc=scenes.GRAVITY)
        sb.box(b, 0.5, 0.5, density=1.0, friction=0.5)
    return sb.build()


def test_gradient_against_finite_differences_of_the_fp64_oracle(gpu_lib):
    """d(mean box x after 30 steps)/d(disk's initial velocity and position),
    adjoint on the GPU against central differences of the FP64 oracle (the
    reference's step in double).  Both solve to convergence (200 velocity and
    30 position iterations), so the Gauss-Seidel order does not matter."""
    sc = _fd_scene()
    steps = 30
    over = dict(regVelocityIters=200, regPositionIters=30, minStillTimeToSleep=1e9, regMinSeparation=-1e-9)
    conf = default_conf(**over)
    boxes = [2, 3, 4]
    g = GpuBatch([sc])
    g.step(deltaTime=0.0)
    g.adjoint_begin(10)
    g.adjoint_forward(steps, conf)
    ybar = np.zeros((sc.n_bodies, 3))
    ybar[boxes, 0] = 1.0 / len(boxes)
    adj = g.adjoint_backward(ybar, None)
    info = g.adjoint_info()
    assert info["replay_mismatches"] == 0 and info["tape_overflows"] == 0, info

    def loss(dvx=0.0, dx=0.0):
        s2 = scenes.Scene(**{f: getattr(sc, f) for f in sc.__dataclass_fields__})
        s2.body_vel = sc.body_vel.astype(np.float64).copy()
        s2.body_pos = sc.body_pos.astype(np.float64).copy()
        s2.body_vel[1, 0] += dvx
        s2.body_pos[1, 0] += dx
        o = oracle.OracleWorld(s2, double=True)
        o.step(deltaTime=0.0)
        for _ in range(steps):
            o.step(**over)
        return float(o.bodies()["pos"][boxes, 0].mean())

    h = 1e-4
    fd_v = (loss(dvx=h) - loss(dvx=-h)) / (2 * h)
    fd_x = (loss(dx=h) - loss(dx=-h)) / (2 * h)
    ad_v, ad_x = float(adj["vel"][1, 0]), float(adj["pos"][1, 0])
    print(f"\nd(mean box x)/d(disk vx): adjoint {ad_v:.6f} fd {fd_v:.6f}; d/d(disk x): adjoint {ad_x:.6f} fd {fd_x:.6f}")
    assert abs(ad_v - fd_v) <= 1e-3 * max(abs(fd_v), 1e-3) + 1e-4
    assert abs(ad_x - fd_x) <= 1e-3 * max(abs(fd_x), 1e-3) + 1e-4


def _chain_scene(n_links=6, disk_vx=6.0, x0=0.0):
    """A chain of 0.2 x 1 m boxes on revolute joints hanging from a static anchor,
    struck by a disk rolling along the ground."""
    sb = scenes.SceneBuilder()
    gnd = sb.body(scenes.STATIC, 0.0, 0.0)
    sb.edge(gnd, (-20.0, 0.0), (40.0, 0.0), friction=0.5)
    top = float(n_links) + 0.6  # the tip link reaches down to 0.6 m, into the disk's path
    anchor = sb.body(scenes.STATIC, x0 + 2.5, top)
    d = sb.body(scenes.DYNAMIC, x0, 0.5, v=(disk_vx, 0.0, 0.0), acc=scenes.GRAVITY)
    sb.disk(d, 0.5, density=1.0, friction=0.5)
    prev = anchor
    for k in range(n_links):
        b = sb.body(scenes.DYNAMIC, x0 + 2.5, top - 0.5 - 1.0 * k, acc=scenes.GRAVITY)
        sb.box(b, 0.1, 0.5, density=1.0, friction=0.5, filt=(2, 0xFFFD, 0, 0))
        sb.revolute(prev, b, (0.0, 0.0) if prev == anchor else (0.0, -0.5), (0.0, 0.5))
        prev = b
    return sb.build()


def test_joint_dot_product_and_replay(gpu_lib):
    """The dot-product test on worlds whose disks strike hanging chains: revolute
    joints' warm start, velocity and position rows and stored impulses, in the
    adjoint and in the tangent, and the joint geometry replayed bit for bit."""
    worlds = [_chain_scene(n_links=4 + k, disk_vx=5.0 + k) for k in range(4)]
    g = GpuBatch(worlds)
    conf = default_conf(minStillTimeToSleep=1e9)
    g.step_n(25, conf)  # the disks reach the chains
    g.adjoint_begin(4)
    g.adjoint_forward(12, conf)
    rng = np.random.default_rng(1)
    dyn = dynamic_mask(worlds)
    n, s = g.n_bodies, g.n_shapes
    ybar_p = rng.standard_normal((n, 3)) * dyn[:, None]
    ybar_v = rng.standard_normal((n, 3)) * dyn[:, None]
    xdot_p = rng.standard_normal((n, 3)) * dyn[:, None] * 1e-2
    xdot_v = rng.standard_normal((n, 3)) * dyn[:, None] * 1e-1
    xdot_f = rng.standard_normal(s) * 1e-2
    adj = g.adjoint_backward(ybar_p, ybar_v)
    tan = g.adjoint_tangent(xdot_p, xdot_v, xdot_f)
    info = g.adjoint_info()
    assert info["replay_mismatches"] == 0, info
    assert info["tape_overflows"] == 0, info
    lhs = float((ybar_p * tan["pos"]).sum() + (ybar_v * tan["vel"]).sum())
    rhs = float((adj["pos"].astype(np.float64) * xdot_p).sum() + (adj["vel"].astype(np.float64) * xdot_v).sum() +
                (adj["friction"].astype(np.float64) * xdot_f).sum())
    scale = max(abs(lhs), abs(rhs), 1e-12)
    print(f"\njoint dot-product test: <ybar, J xdot> = {lhs:.9e}, <J^T ybar, xdot> = {rhs:.9e}, "
          f"rel diff {abs(lhs - rhs) / scale:.2e}")
    assert abs(lhs - rhs) <= 1e-4 * scale
    g.adjoint_end()


def test_joint_gradient_against_finite_differences_of_the_fp64_oracle(gpu_lib):
    """d(chain tip x after 40 steps)/d(disk's initial vx and x): the disk strikes
    the chain's tip, so the gradient runs through the contact and back up the
    joints.  Adjoint on the GPU against central differences of the FP64 oracle,
    both solved to convergence.  (Perturbing a link's own state instead shows the
    colour-order difference of the position iterations, which do not converge
    in 30 iterations: the GPU forward's own finite difference then agrees with
    the adjoint, not with the oracle's.)"""
    sc = _chain_scene(n_links=4, disk_vx=6.0)
    steps = 40
    over = dict(regVelocityIters=200, regPositionIters=30, minStillTimeToSleep=1e9, regMinSeparation=-1e-9)
    conf = default_conf(**over)
    tip, disk = sc.n_bodies - 1, 2
    g = GpuBatch([sc])
    g.step(deltaTime=0.0)
    g.adjoint_begin(10)
    g.adjoint_forward(steps, conf)
    ybar = np.zeros((sc.n_bodies, 3))
    ybar[tip, 0] = 1.0
    adj = g.adjoint_backward(ybar, None)
    info = g.adjoint_info()
    assert info["replay_mismatches"] == 0 and info["tape_overflows"] == 0, info

    def loss(dvx=0.0, dx=0.0):
        s2 = scenes.Scene(**{f: getattr(sc, f) for f in sc.__dataclass_fields__})
        s2.body_vel = sc.body_vel.astype(np.float64).copy()
        s2.body_pos = sc.body_pos.astype(np.float64).copy()
        s2.body_vel[disk, 0] += dvx
        s2.body_pos[disk, 0] += dx
        o = oracle.OracleWorld(s2, double=True)
        o.step(deltaTime=0.0)
        for _ in range(steps):
            o.step(**over)
        return float(o.bodies()["pos"][tip, 0])

    h = 1e-4
    fd_v = (loss(dvx=h) - loss(dvx=-h)) / (2 * h)
    fd_x = (loss(dx=h) - loss(dx=-h)) / (2 * h)
    ad_v, ad_x = float(adj["vel"][disk, 0]), float(adj["pos"][disk, 0])
    print(f"\nd(tip x)/d(disk vx): adjoint {ad_v:.6f} fd {fd_v:.6f}; d/d(disk x): adjoint {ad_x:.6f} fd {fd_x:.6f}")
    assert abs(ad_v - fd_v) <= 1e-3 * max(abs(fd_v), 1e-3) + 1e-4
    assert abs(ad_x - fd_x) <= 1e-3 * max(abs(fd_x), 1e-3) + 1e-4


# ---- the differentiable workload: 64 pushing worlds, checkpoint every 16 -------
PUSH_CONF = dict(regVelocityIters=200, regPositionIters=30, minStillTimeToSleep=1e9, regMinSeparation=-1e-9)


def _push_targets(n):
    rng = np.random.default_rng(2)
    return np.stack([rng.uniform(10, 30, n), rng.uniform(0, 2, n)], 1)


def _push_loss(pos, targets, k):
    m = np.asarray(pos, np.float64)[2:34, :2].mean(0)  # ground, disk, then the 32 boxes
    return float(((m - targets[k]) ** 2).sum())


@pytest.mark.parametrize("steps", [60, 240])
def test_push_workload_gradients_against_fp64_finite_differences(gpu_lib, steps):
    """The differentiable workload: 64 worlds (a disk pushing 32 boxes on a ground,
    all with friction mu, seed 2), checkpoint every 16 steps, loss = squared
    distance of each world's mean box centre from its target in [10,30]x[0,2].
    d(loss)/d(disk initial velocity x, y) and d(loss)/d(mu) from StepAdjoint on
    the whole batch.

    mu is every shape's friction, so MixFriction (sqrt(f1 f2), Contact.hpp:57)
    gives mu for every contact and d(loss)/d(mu) is the sum of the adjoint's
    d(loss)/d(shape friction) over the world's shapes.

    Solved to convergence (200 velocity, 30 position iterations, no sleep).  Two
    checks:

    1. The adjoint (float reverse pass) against the FP64 tangent of the same
       forward (forward mode along the GPU's own trajectory): every world and
       parameter.  Over 60 steps within 1e-3; over 240 steps the reverse pass's
       float rounding grows with the window in a few worlds, so there 90 % of the
       pairs are held to 1e-3, and a derivative that grows beyond 1e6 (a chaotic
       world, where the forward tangent itself explodes) is reported, not checked.

    2. Against central differences (h = 1e-4) of the FP64 oracle, which replays
       step by step the Gauss-Seidel order the GPU swept
       (prgpu_download_sweep_order): the position solver's fixed points are not
       unique, and over hundreds of steps the order would otherwise dominate.
       The loss is only piecewise smooth (contacts begin and end, friction
       switches between sticking and sliding), and the FP64 trajectory takes its
       own pieces: it is compared where it takes the GPU's (the same number of
       touching contacts in every step) and where the central differences at h
       and h/2 agree within 1e-5 relative.  On a smooth piece they differ by
       O(h^2) and by the FP64 rounding of the loss over 2h, both below 1e-8
       here; a larger gap means a piece boundary (a stick-slip switch, say)
       within h.  Every pair that counts must agree with the adjoint within 1e-3
       relative; every 4th world is checked (16 of 64)."""
    worlds = scenes.push_worlds(64, seed=2)
    targets = _push_targets(64)
    conf = default_conf(**PUSH_CONF)
    # the forward's sweep order and touching contacts, step by step (the step is
    # deterministic: the adjoint's own forward takes the same path)
    rec = GpuBatch(worlds)
    orders, touching = [], np.zeros((steps, len(worlds)), np.int64)
    sb = np.asarray(rec.shape_base, np.int64)
    for s in range(steps):
        rec.step(conf)
        o = rec.sweep_order().astype(np.int64)
        w = np.searchsorted(sb, o[:, 1], side="right") - 1
        loc = o.copy()
        loc[:, 1] -= sb[w]
        loc[:, 2] -= sb[w]
        orders.append([loc[w == k] for k in range(len(worlds))])
        c = rec.contacts()
        cw = np.searchsorted(sb, c["proxy"][:, 0], side="right") - 1
        touching[s] = np.bincount(cw[c["touching"] != 0], minlength=len(worlds))
    g = GpuBatch(worlds)
    g.adjoint_begin(16)
    g.adjoint_forward(steps, conf)
    b = g.bodies()
    np.testing.assert_array_equal(b["pos"], rec.bodies()["pos"])
    ybar = np.zeros((g.n_bodies, 3))
    for k in range(len(worlds)):
        lo = int(g.body_base[k])
        m = b["pos"][lo + 2:lo + 34, :2].astype(np.float64).mean(0)
        ybar[lo + 2:lo + 34, :2] = 2.0 * (m - targets[k]) / 32.0
    adj = g.adjoint_backward(ybar, None)
    info = g.adjoint_info()
    assert info["replay_mismatches"] == 0 and info["tape_overflows"] == 0, info
    # the same derivatives by the FP64 tangent, all worlds at once
    tan = {}
    for name in ("vx", "vy", "mu"):
        dv, df = np.zeros((g.n_bodies, 3)), np.zeros(g.n_shapes)
        for k in range(len(worlds)):
            if name == "mu":
                df[int(g.shape_base[k]):int(g.shape_base[k + 1])] = 1.0
            else:
                dv[int(g.body_base[k]) + 1, 0 if name == "vx" else 1] = 1.0
        tan[name] = g.adjoint_tangent(None, dv, df)["pos"]
    g.adjoint_end()

    def adjoint(k):
        lo, hi = int(g.body_base[k]), int(g.shape_base[k])
        return {"vx": float(adj["vel"][lo + 1, 0]), "vy": float(adj["vel"][lo + 1, 1]),
                "mu": float(adj["friction"][hi:int(g.shape_base[k + 1])].astype(np.float64).sum())}

    rels, nonfinite, exploding = [], [], []
    for k in range(len(worlds)):
        lo, hi = int(g.body_base[k]), int(g.body_base[k + 1])
        ad = adjoint(k)
        for name in ("vx", "vy", "mu"):
            t = float((ybar[lo:hi] * tan[name][lo:hi]).sum())
            if not np.isfinite(t) or abs(t) > 1e6:
                # the forward map's derivative itself explodes (chaotic growth over
                # the window): beyond float range for the reverse pass, no check
                exploding.append((k, name, t))
                continue
            if not np.isfinite(ad[name]):
                nonfinite.append((k, name, ad[name], t))
            rels.append(abs(ad[name] - t) / max(abs(t), 1e-3))
    assert not nonfinite, nonfinite
    rels = np.asarray(rels)
    print(f"\n{steps} steps: adjoint vs FP64 tangent, worst rel {rels.max():.1e}, "
          f"within 1e-3: {np.mean(rels <= 1e-3):.1%}; exploding derivatives: {exploding}")
    if steps == 60:
        assert rels.max() <= 1e-3 and not exploding
    else:
        assert np.mean(rels <= 1e-3) >= 0.9

    def run(k, dvx=0.0, dvy=0.0, dmu=0.0, count=None):
        sc = worlds[k]
        s2 = scenes.Scene(**{f: getattr(sc, f) for f in sc.__dataclass_fields__})
        s2.body_vel = sc.body_vel.astype(np.float64).copy()
        s2.body_vel[1, 0] += dvx
        s2.body_vel[1, 1] += dvy
        s2.shape_friction = sc.shape_friction.astype(np.float64) + dmu
        o = oracle.OracleWorld(s2, double=True)
        for s in range(steps):
            o.set_solve_order(orders[s][k])
            o.step(**PUSH_CONF)
            if count is not None:
                count.append(int(o.contacts()["touching"].sum()))
        return _push_loss(o.bodies()["pos"], targets, k)

    h = 1e-4
    checked, report, skipped = {"vx": 0, "vy": 0, "mu": 0}, [], []
    for k in range(0, 64, 4):
        seq = []
        run(k, count=seq)
        if not np.array_equal(seq, touching[:, k]):
            skipped.append(k)  # the FP64 run takes other pieces: no common derivative
            continue
        ad = adjoint(k)
        for name, kw in (("vx", "dvx"), ("vy", "dvy"), ("mu", "dmu")):
            fd = (run(k, **{kw: h}) - run(k, **{kw: -h})) / (2 * h)
            fd2 = (run(k, **{kw: h / 2}) - run(k, **{kw: -h / 2})) / h
            if abs(fd - fd2) > 1e-5 * max(abs(fd), 1e-3):
                continue  # not smooth at this point: no derivative to compare
            checked[name] += 1
            rel = abs(ad[name] - fd) / max(abs(fd), 1e-3)
            report.append((k, name, ad[name], fd, rel))
    print(f"{steps} steps, smooth pairs checked {checked}; worlds whose FP64 run took other pieces: {skipped}")
    for k, name, a, f, r in report:
        print(f"  world {k:2d} d/d{name}: adjoint {a:.6g} fd {f:.6g} rel {r:.1e}")
    bad = [r for r in report if r[4] > 1e-3]
    assert not bad, bad
    if steps == 60:
        assert checked["vx"] >= 6 and checked["vy"] >= 6 and checked["mu"] >= 2, checked
    else:
        assert checked["vx"] + checked["vy"] >= 2, checked


def test_window_in_pieces_matches_one_call(gpu_lib):
    """The forward pass records the window's last segment as it runs it, and the
    backward pass uses those tapes instead of running that segment again.  The
    reverse pass sums its body adjoints in FP64, so its gradients do not depend
    on the order of its atomics: a window run in one forward call, in several
    (segments split across calls, the recorded segment continued by a later call,
    the last segment partial), a second backward pass over the same window (every
    segment recomputed) and a backward pass after a tangent pass (which records
    over the tapes) all give the same position and velocity gradients, bit for
    bit."""
    worlds = scenes.push_worlds(8, seed=2)
    conf = default_conf(minStillTimeToSleep=1e9)
    dyn = dynamic_mask(worlds)
    rng = np.random.default_rng(1)
    n = int(dyn.size)
    ybar_p = rng.standard_normal((n, 3)) * dyn[:, None]
    ybar_v = rng.standard_normal((n, 3)) * dyn[:, None]

    def window(pieces, steps_before=40):
        g = GpuBatch(worlds)
        g.step_n(steps_before, conf)
        g.adjoint_begin(16)
        for k in pieces:
            g.adjoint_forward(k, conf)
        return g

    def check_same(a, b, what):
        np.testing.assert_array_equal(a["pos"], b["pos"], err_msg=what)
        np.testing.assert_array_equal(a["vel"], b["vel"], err_msg=what)

    for total, splits in ((100, ([37, 50, 13], [84, 16])), (95, ([90, 5],))):
        g = window([total])
        one = g.adjoint_backward(ybar_p, ybar_v)
        assert np.abs(one["vel"]).max() > 0.0
        check_same(one, g.adjoint_backward(ybar_p, ybar_v), f"{total} steps: second backward pass")
        g.adjoint_tangent(ybar_p * 1e-3, ybar_v * 1e-3)
        check_same(one, g.adjoint_backward(ybar_p, ybar_v), f"{total} steps: backward after the tangent")
        info = g.adjoint_info()
        assert info["steps"] == total and info["replay_mismatches"] == 0 and info["tape_overflows"] == 0, info
        g.adjoint_end()
        for pieces in splits:
            h = window(pieces)
            check_same(one, h.adjoint_backward(ybar_p, ybar_v), f"forward calls {pieces}")
            info = h.adjoint_info()
            assert info["replay_mismatches"] == 0 and info["tape_overflows"] == 0, info
            h.adjoint_end()
