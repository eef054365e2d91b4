"""Runs scenes through the PlayRho reference compiled from source (oracle/ref).

Available where the reference sources have been staged into oracle/_ref/src
(``make -C oracle/ref stage PLAYRHO_REFERENCE=<checkout>``; git-ignored, never
committed): the binaries live in oracle/_ref/ and are built from that copy by
``make -C oracle/ref``.  Used to check the oracle and as the CPU baseline;
never part of the shipped library.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
REF_SRC = os.path.join(REF_DIR, "src")  # the staged copy of the reference


def staged() -> bool:
    return os.path.isdir(os.path.join(REF_SRC, "Library", "source"))


def available(double: bool = False) -> bool:
    return os.path.exists(driver_path(double)) or staged()


def driver_path(double: bool = False) -> str:
    return os.path.join(REF_DIR, "ref_driver_f64" if double else "ref_driver_f32")


def ensure_built(double: bool = False) -> str:
    path = driver_path(double)
    if staged() or not os.path.exists(path):
        # make relinks the driver when oracle/ref/ref_driver.cpp changed
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"-j{os.cpu_count() or 8}",
                        "f64" if double else "f32"], check=True)
    return path


def ensure_bench_built() -> str:
    """Builds the multi-world timing driver (oracle/ref/ref_bench.cpp)."""
    path = os.path.join(REF_DIR, "ref_bench_f32")
    if staged() or not os.path.exists(path):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"-j{os.cpu_count() or 8}", "bench"],
                       check=True)
    return path


def _f(tok: str) -> float:
    return float.fromhex(tok)


def run(scene_text: str, steps, double: bool = False, timeout: float = 600.0):
    """Runs ``steps`` (an int or a list of ints, dumping after each) and parses the dumps."""
    path = ensure_built(double)
    seq = [steps] if isinstance(steps, int) else list(steps)
    cmd = scene_text + "".join(f"step {n}\ndump\n" for n in seq)
    res = subprocess.run([path], input=cmd, capture_output=True, text=True, timeout=timeout, check=True)
    dumps, cur, events, calls, complete = [], None, [], [], 1
    for line in res.stdout.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "ev":
            events.append(tuple(int(x) for x in t[1:4]))
        elif t[0] == "solve":
            calls.append(tuple(int(x) for x in t[1:6]) + tuple(_f(x) for x in t[6:10]))
        elif t[0] == "complete":
            complete = int(t[1])
        elif t[0] == "stats":
            cur = {"stats": [int(x) for x in t[1:10]] + [_f(x) for x in t[10:12]],
                   "bodies": [], "proxies": [], "contacts": [], "events": events, "solve_calls": calls,
                   "complete": complete}
            events, calls = [], []
        elif t[0] == "toistats":
            cur["toistats"] = [int(x) for x in t[1:15]] + [_f(x) for x in t[15:17]]
        elif t[0] == "body":
            cur["bodies"].append([_f(x) for x in t[2:15]] + [int(t[15])])
        elif t[0] == "proxy":
            cur["proxies"].append([int(x) for x in t[1:5]] + [_f(x) for x in t[5:9]])
        elif t[0] == "contact":
            ints = [int(x) for x in t[1:14]]
            floats = [_f(x) for x in t[14:26]]
            feats = [int(x) for x in t[26:34]]
            cur["contacts"].append((ints, floats, feats))
        elif t[0] == "end":
            dumps.append(_finish(cur, double))
    return dumps


def run_rays(scene_text: str, steps: int, rays, double: bool = False, timeout: float = 600.0):
    """Steps the scene ``steps`` times, then casts each ray (x1, y1, x2, y2,
    maxFraction) through RayCast(World, ...) with a callback answering ResetRay;
    returns per ray the list of hits (shape, point x, point y, normal x, normal y)
    in the reference's tree order."""
    path = ensure_built(double)
    cmd = scene_text + f"step {int(steps)}\n" + "".join("ray " + " ".join(repr(float(v)) for v in r) + "\n"
                                                        for r in rays)
    res = subprocess.run([path], input=cmd, capture_output=True, text=True, timeout=timeout, check=True)
    out, cur = [], []
    for line in res.stdout.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "rayhit":
            cur.append((int(t[1]),) + tuple(_f(x) for x in t[2:6]))
        elif t[0] == "rayend":
            out.append(cur)
            cur = []
    return out


def _finish(d, double):
    npr = np.float64 if double else np.float32
    b = np.asarray([x[:13] for x in d["bodies"]], dtype=np.float64).reshape(-1, 13)
    aw = np.asarray([x[13] for x in d["bodies"]], dtype=np.int32)
    bodies = {"pos": b[:, 0:3].astype(npr), "vel": b[:, 3:6].astype(npr), "xf": b[:, 6:10].astype(npr),
              "inv_mass": b[:, 10].astype(npr), "inv_rot_inertia": b[:, 11].astype(npr),
              "under_active": b[:, 12].astype(npr), "awake": aw}
    pr = d["proxies"]
    proxies = {"bsc": np.asarray([p[1:4] for p in pr], dtype=np.int32).reshape(-1, 3),
               "aabb": np.asarray([p[4:8] for p in pr], dtype=np.float64).astype(npr).reshape(-1, 4)}
    cs = d["contacts"]
    n = len(cs)
    io = np.asarray([c[0] for c in cs], dtype=np.int32).reshape(n, 13)
    fo = np.asarray([c[1] for c in cs], dtype=np.float64).astype(npr).reshape(n, 12)
    ft = np.asarray([c[2] for c in cs], dtype=np.int32).reshape(n, 8)
    contacts = {"id": io[:, 1], "proxy": io[:, 2:4], "bsc_a": io[:, 4:7], "bsc_b": io[:, 7:10],
                "touching": io[:, 10], "type": io[:, 11], "count": io[:, 12], "local_normal": fo[:, 0:2],
                "local_point": fo[:, 2:4], "points": fo[:, 4:12].reshape(n, 2, 4),
                "features": ft.reshape(n, 2, 4)}
    return {"stats": d["stats"], "toistats": d.get("toistats"), "bodies": bodies, "proxies": proxies,
            "contacts": contacts, "events": d["events"], "solve_calls": d["solve_calls"], "complete": d["complete"]}
