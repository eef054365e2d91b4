"""The C++ host layer (prgpu::HostWorld, playrho_gb300/host/) driven by a small
C++ program in the style of a PlayRho application, against the batch API.

CPU tests compile the program and check the pool bookkeeping and the error
path without a GPU; GPU tests check that worlds built through HostWorld step
bit for bit like the same scene given to the batch API, including SetBody
between steps.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from playrho_gb300 import build, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "playrho_gb300")


@pytest.fixture(scope="module")
def checker():
    build.build()
    out = os.path.join(tempfile.mkdtemp(prefix="hw_"), "host_world_check")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(PKG, "host"),
           os.path.join(ROOT, "tests", "host_world_check.cpp"), "-L" + PKG, "-lprgpu_host", "-lprgpu",
           "-Wl,-rpath," + PKG, "-o", out]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return out


def run(checker, text):
    return subprocess.run([checker], input=text, capture_output=True, text=True, timeout=600)


def parse_dump(out):
    rows = [l.split() for l in out.splitlines() if l.startswith("b ")]
    idx = np.array([int(r[1]) for r in rows])
    vals = np.array([[float.fromhex(x) for x in r[2:8]] for r in rows], dtype=np.float64).astype(np.float32)
    return idx, vals


def test_pools_without_gpu(checker):
    sc = scenes.pyramid(rows=3)
    res = run(checker, scenes.scene_text(sc) + "dump\ndestroy_body 1\ndump\n")
    assert res.returncode == 0, res.stderr
    idx, vals = parse_dump(res.stdout)
    n = sc.n_bodies
    # first dump: every body with its initial origin; second: body 1 gone
    assert list(idx[:n]) == list(range(n)) and 1 not in list(idx[n:]) and len(idx) == 2 * n - 1
    np.testing.assert_array_equal(vals[:n, :2], sc.body_pos[:, :2].astype(np.float32))


def test_step_without_gpu_reports_status(checker):
    from playrho_gb300.gpu import gpu_available

    if gpu_available():
        pytest.skip("a GPU is present")
    res = run(checker, scenes.scene_text(scenes.pyramid(rows=2)) + "step 1\n")
    # status PRGPU_ENOTREADY (5) surfaces as a HostWorld error, exit 10 + 5
    assert res.returncode == 15, (res.returncode, res.stderr)
    assert "prgpu_world_create" in res.stderr


def _shapes_by_body(sc):
    return bool(np.all(np.diff(sc.shape_body) >= 0))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["pile", "chains", "joint_zoo"])
def test_host_world_steps_like_the_batch(checker, gpu_lib, kind):
    from playrho_gb300.gpu import GpuBatch

    rng = np.random.default_rng(21)
    if kind == "pile":
        sc = scenes.pile(120, rng, width=5.0)
    elif kind == "chains":
        sc = scenes.chains_world(rng, n_free=60, n_chains=3, links=6)
    else:
        sc = scenes.joint_zoo(rng, per_kind=2, n_disks=10)
    assert _shapes_by_body(sc)  # proxies in the same order on both paths
    res = run(checker, scenes.scene_text(sc) + "step 90\ndump\n")
    assert res.returncode == 0, res.stderr
    _, vals = parse_dump(res.stdout)
    g = GpuBatch([sc])
    for _ in range(90):
        g.step()
    b = g.bodies()
    np.testing.assert_array_equal(vals[:, 0:2], b["xf"][:, 0:2])
    np.testing.assert_array_equal(vals[:, 2], b["pos"][:, 2])
    np.testing.assert_array_equal(vals[:, 3:6], b["vel"])


@pytest.mark.gpu
def test_host_world_set_body_between_steps(checker, gpu_lib):
    """SetBody of a position between steps takes the in-place upload path."""
    from playrho_gb300.gpu import GpuBatch

    rng = np.random.default_rng(22)
    sc = scenes.pile(80, rng, width=5.0)
    disks = [i for i in range(sc.n_bodies)
             if sc.body_type[i] == scenes.DYNAMIC and sc.shape_kind[list(sc.shape_body).index(i)] == 0]
    bi = disks[0]
    g = GpuBatch([sc])
    for _ in range(30):
        g.step()
    b = g.bodies()
    nx, ny = np.float32(b["xf"][bi, 0] + 0.25), np.float32(b["xf"][bi, 1] + 2.0)
    text = scenes.scene_text(sc) + f"step 30\nteleport {bi} {float(nx).hex()} {float(ny).hex()}\nstep 30\ndump\n"
    res = run(checker, text)
    assert res.returncode == 0, res.stderr
    _, vals = parse_dump(res.stdout)
    # the batch: same teleport (a disk's centre of mass is its origin)
    pos = b["pos"][bi:bi + 1].copy()
    pos[0, 0], pos[0, 1] = nx, ny
    g.set_body_states(pos=pos, vel=b["vel"][bi:bi + 1].copy(), first=bi)
    for _ in range(30):
        g.step()
    b2 = g.bodies()
    np.testing.assert_array_equal(vals[:, 0:2], b2["xf"][:, 0:2])
    np.testing.assert_array_equal(vals[:, 3:6], b2["vel"])
