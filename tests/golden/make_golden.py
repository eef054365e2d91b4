"""Generates the golden fixtures of the oracle from the PlayRho reference itself.

Runs each scene through the reference compiled from source (oracle/ref, built
with `make -C oracle/ref`) and stores, per fixture, the scene arrays and the
reference's bodies, contacts and step statistics after the listed steps, with
FP32 values kept bit-exact.  Needs the reference sources staged into
oracle/_ref/src (``make -C oracle/ref stage PLAYRHO_REFERENCE=<checkout>``);
the fixtures it writes are what the oracle is checked against wherever the
sources are absent.

    python tests/golden/make_golden.py [fixture names]
"""
from __future__ import annotations

import dataclasses
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refdriver  # noqa: E402
from playrho_gb300 import scenes  # noqa: E402


def helloworld_scene():
    """HelloWorld/HelloWorld.cpp: a 50x10 half-extent ground box at (0,-10) and a
    1 m disk dropped from (0,4) with the reference's EarthlyGravity (-9.8f)."""
    sb = scenes.SceneBuilder()
    g = sb.body(scenes.STATIC, 0.0, -10.0)
    sb.box(g, 50.0, 10.0)
    b = sb.body(scenes.DYNAMIC, 0.0, 4.0, acc=(0.0, float(np.float32(-9.8)), 0.0))
    sb.disk(b, 1.0)
    return sb.build()


def cases():
    return {
        "pyramid20": (scenes.pyramid(), [1, 10, 60, 200, 600], {}),
        "pile300_seed5": (scenes.pile(300, np.random.default_rng(5)), [1, 100, 300], {}),
        "box2000_seed0": (scenes.large_box(2000, size=60.0, seed=0), [1, 50], {}),
        "chains_seed3": (scenes.chains_world(np.random.default_rng(3), n_free=200, n_chains=4, links=8),
                         [1, 100], {}),
        "helloworld": (helloworld_scene(), list(range(1, 61)), {}),
        # time-of-impact phase on (StepConf::doToi, the reference's default)
        "toi_bullets60_seed3": (scenes.bullets(60, np.random.default_rng(3)), [1, 5, 30, 90], {"doToi": 1}),
        "toi_pile200_seed11": (scenes.pile(200, np.random.default_rng(11)), [1, 60, 180, 300], {"doToi": 1}),
        # distance, rope, weld, friction and motor joints side by side
        "joint_zoo_seed7": (scenes.joint_zoo(np.random.default_rng(7)), [1, 60, 180], {}),
    }


def save(name, scene, steps, conf, double=False):
    dumps = refdriver.run(scenes.scene_text(scene, conf), [steps[0]] + [b - a for a, b in zip(steps, steps[1:])],
                          double=double)
    out = {f"scene_{k}": v for k, v in dataclasses.asdict(scene).items()}
    out["steps"] = np.asarray(steps, np.int32)
    for k, v in conf.items():
        out[f"conf_{k}"] = np.asarray(v)
    for i, d in enumerate(dumps):
        b, c = d["bodies"], d["contacts"]
        out[f"d{i}_pos"] = b["pos"]
        out[f"d{i}_vel"] = b["vel"]
        out[f"d{i}_awake"] = b["awake"]
        out[f"d{i}_stats"] = np.asarray(d["stats"][:9], np.int64)
        if conf.get("doToi"):
            out[f"d{i}_toistats"] = np.asarray(d["toistats"][:14], np.int64)
        if name != "helloworld" or i in (0, 29, 59):
            out[f"d{i}_c_proxy"] = c["proxy"]
            out[f"d{i}_c_count"] = c["count"]
            out[f"d{i}_c_type"] = c["type"]
            out[f"d{i}_c_features"] = c["features"]
            out[f"d{i}_c_points"] = c["points"]
            out[f"d{i}_c_touching"] = c["touching"]
    path = os.path.join(HERE, f"ref_{name}{'_f64' if double else ''}.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


def main(names=None):
    """Writes every fixture, or only those named on the command line."""
    for name, (scene, steps, conf) in cases().items():
        if not names or name in names:
            save(name, scene, steps, conf)
    if not names or "pile300_seed5_f64" in names:
        save("pile300_seed5", scenes.pile(300, np.random.default_rng(5)), [1, 100, 300], {}, double=True)
    if not names or "toi_bullets60_seed3_f64" in names:
        save("toi_bullets60_seed3", scenes.bullets(60, np.random.default_rng(3)), [1, 30, 90], {"doToi": 1},
             double=True)


if __name__ == "__main__":
    main(sys.argv[1:])
