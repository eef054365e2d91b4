"""The C++ drop-in: playrho::d2::World{GpuWorld{}} compiled against the
reference's own headers and library (the reference's HelloWorld with the World
constructed over GpuWorld), where the reference sources are available.

Set-up runs through PlayRho's World API into GpuWorld (CreateShape, CreateBody
with BodyConf::Use(shape), GetBodies, GetInvMass ...); Step reaches the GPU
library, which without a GPU answers PRGPU_ENOTREADY, surfaced as an exception.
On a GPU machine (the -m gpu test) the same program steps the world on the GPU.
The reference's headers and library come from the staged copy of its sources
(oracle/_ref/src, oracle/ref/Makefile), built on the machine that runs the test.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

from playrho_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "playrho_gb300")
REF = os.path.join(ROOT, "oracle", "_ref", "src")  # the staged reference (oracle/ref/Makefile stage)
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "f32", "libPlayRho.a")
REF_GEN = os.path.join(ROOT, "oracle", "_ref", "f32", "gen")


_EXE = []


def _compile():
    if _EXE:
        return _EXE[0]
    if not os.path.isdir(os.path.join(REF, "Library", "include")):
        pytest.skip("reference sources not staged here (make -C oracle/ref stage)")
    if not os.path.exists(REF_LIB):
        res = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"-j{os.cpu_count() or 8}",
                              "f32"], capture_output=True, text=True)
        if res.returncode or not os.path.exists(REF_LIB):
            pytest.skip("reference library could not be built here")
    build.build()
    out = os.path.join(tempfile.mkdtemp(prefix="gw_"), "gpuworld_check")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O1", "-std=c++17", "-ffp-contract=off", "-w", "-I" + REF_GEN,
           "-I" + os.path.join(REF, "Library", "include"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(PKG, "host"), os.path.join(ROOT, "tests", "gpuworld_check.cpp"),
           os.path.join(PKG, "host", "GpuWorld.cpp"), REF_LIB, "-L" + PKG, "-lprgpu_host", "-lprgpu",
           "-Wl,-rpath," + PKG, "-o", out]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    _EXE.append(out)
    return out


def test_world_over_gpuworld_builds_and_runs():
    exe = _compile()
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    lines = dict(l.split(" ", 1) for l in res.stdout.splitlines() if " " in l)
    assert lines["bodies"] == "2"
    assert lines["shapes"] == "2"
    assert lines["type"] == "2"  # BodyType::Dynamic
    # a disk of density 0 gets the reference's default mass of 1 kg and no rotational inertia
    inv_mass, inv_rot = (float.fromhex(x) for x in lines["mass"].split())
    assert inv_mass == 1.0 and inv_rot == 0.0
    # one joint of each kind reaches the GPU side with its kind and parameters
    joints = [l.split()[1:] for l in res.stdout.splitlines() if l.startswith("joint ")]
    assert [int(j[0]) for j in joints] == list(range(10))  # prgpu_joint_kind order
    extra = {int(j[0]): [float.fromhex(x) for x in j[4:11]] for j in joints}
    flags = {int(j[0]): [int(x) for x in j[11:15]] for j in joints}
    assert all(float.fromhex(j[2]) == 0.25 and float.fromhex(j[3]) == 0.5 for j in joints[:5])
    assert int(joints[2][1]) == 1 and int(joints[1][1]) == 0  # collideConnected
    assert extra[1][:3] == [1.5, 4.0, 0.5]
    assert extra[2][:1] == [2.5]
    assert extra[3][:3] == [0.25, 2.0, 0.75]
    assert extra[4][:2] == [3.0, 1.5]
    assert extra[5][:6] == [1.0, -0.5, 0.125, 10.0, 5.0, 0.25]
    assert extra[6] == [0.0, 1.0, 0.5, -1.0, 2.0, 3.0, 7.0] and flags[6][:2] == [1, 1]
    assert extra[7][:6] == [0.0, 1.0, -2.0, 6.0, 4.0, 0.5] and flags[7][:2] == [0, 1]
    assert extra[8] == [-1.0, 5.0, 2.0, 5.0, 4.0, 3.0, 1.5] and int(joints[8][1]) == 1  # pulley collides
    assert extra[9][:5] == [3.0, 4.0, 9.0, 3.0, 0.25]
    assert flags[9][2] == flags[9][3] == flags[0][3]  # the target joint holds body B only
    assert any(l.startswith("joint_rejected ") for l in res.stdout.splitlines())  # a gear without joints
    assert lines["gear"] == "10 0 6 2 1"  # GetGearJointConf's gear reaches the GPU side with its joints
    from playrho_gb300.gpu import gpu_available

    if not gpu_available():
        assert res.returncode == 3
        assert "prgpu_world_create" in lines.get("error", "")


@pytest.mark.gpu
def test_helloworld_over_gpuworld_steps_on_the_gpu(gpu_lib):
    """The reference's HelloWorld with World{GpuWorld{}} (default StepConf, so the
    time-of-impact phase is on): its 60 printed lines equal the reference's
    HelloWorld/ExpectedOutput.txt, and the disk's location after every step equals,
    bit for bit, the oracle's (pinned to the reference with the time-of-impact
    phase on) on the same scene."""
    import numpy as np

    from oracle import oracle
    from playrho_gb300 import scenes

    exe = _compile()
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    steps = [l.split()[1:] for l in res.stdout.splitlines() if l.startswith("step ")]
    assert len(steps) == 60
    xya = [[float.fromhex(v) for v in s[1:]] for s in steps]
    # HelloWorld prints each value with std::setw(5) and 2 fixed decimals
    printed = ["".join("%5.2f" % v for v in row) for row in xya]
    with open(os.path.join(REF, "HelloWorld", "ExpectedOutput.txt")) as f:
        expected = [l.rstrip("\n") for l in f if l.strip()]
    assert printed == expected[:60]
    # HelloWorld/HelloWorld.cpp: a 50x10 half-extent ground box at (0,-10), a 1 m
    # disk dropped from (0,4) with EarthlyGravity (-9.8f)
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, -10.0)
    sb.box(g, 50.0, 10.0)
    b = sb.body(scenes.DYNAMIC, 0.0, 4.0, acc=(0.0, float(np.float32(-9.8)), 0.0))
    sb.disk(b, 1.0)
    ow = oracle.OracleWorld(sb.build())
    for i in range(60):
        ow.step(doToi=1)
        ref = ow.bodies()["xf"][1]
        assert np.float32(xya[i][0]) == ref[0] and np.float32(xya[i][1]) == ref[1], (i, xya[i], ref)

    # The same program runs one scenario through the reference's own World{} and
    # through World{GpuWorld{}} with identical calls: listener calls, the step at
    # which the box's contact appears (and that its ID keeps naming it), and the
    # box's path with SetContact's tangent speed, friction and disabling.
    def lines(tag, kind):
        return [l.split()[2:] for l in res.stdout.splitlines() if l.startswith(f"{tag} {kind} ")]

    assert lines("gpu", "event") == lines("ref", "event") and len(lines("ref", "event")) >= 2
    assert lines("gpu", "id") == lines("ref", "id") and not lines("gpu", "id_changed")
    gp, rp = lines("gpu", "pos"), lines("ref", "pos")
    assert len(gp) == len(rp) == 60
    for g, r in zip(gp, rp):
        gv, rv = [float.fromhex(x) for x in g[1:]], [float.fromhex(x) for x in r[1:]]
        assert np.allclose(gv, rv, rtol=0, atol=1e-5), (g[0], gv, rv)
    assert float.fromhex(rp[43][1]) > 0.5  # the conveyor moved the box
    assert float.fromhex(rp[59][2]) < 0.3  # once disabled, the contact no longer holds it
    # The scenario again without the time-of-impact phase (whose own listener
    # calls GpuWorld does not make): every listener call, in order (Begin/End,
    # PreSolve, PostSolve), and the pre- and post-solve arguments: point counts
    # and iteration arguments exactly, impulses within 1e-4.
    assert lines("gnt", "call") == lines("rnt", "call")
    for kind, head in (("pre", 4), ("post", 5)):
        gl, rl = lines("gnt", kind), lines("rnt", kind)
        assert len(gl) == len(rl) > 20, kind
        for g, r in zip(gl, rl):
            assert g[:head] == r[:head], (kind, g, r)
            gv, rv = [float.fromhex(x) for x in g[head:]], [float.fromhex(x) for x in r[head:]]
            assert np.allclose(gv, rv, rtol=1e-4, atol=1e-4), (kind, g, r)
    # Multi-child shapes through the drop-in: a chain terrain and MultiShapeConf
    # bodies.  Mass data as the reference's (it computes it; the GPU takes it),
    # the contacts at steps 1, 10, 20 and 30 by (shape, child) pairs and touching
    # state, and the bodies' paths within 2e-3 over the 30 steps (the GPU sweeps
    # each body's contacts with the terrain's edges in colour order, the reference
    # in island order; over longer runs the tumbling bodies' paths part).
    assert lines("gpu", "tmass") == lines("ref", "tmass") and len(lines("ref", "tmass")) == 3
    assert lines("gpu", "tcontact") == lines("ref", "tcontact")
    assert any(int(x[2]) > 0 or int(x[4]) > 0 for x in lines("ref", "tcontact"))  # children past the first touch
    gp, rp = lines("gpu", "tpos"), lines("ref", "tpos")
    assert len(gp) == len(rp) == 18
    for g, r in zip(gp, rp):
        gv, rv = [float.fromhex(x) for x in g[2:]], [float.fromhex(x) for x in r[2:]]
        assert g[:2] == r[:2] and np.allclose(gv, rv, rtol=0, atol=2e-3), (g, r)
