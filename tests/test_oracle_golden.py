"""The CPU oracle against fixtures produced by the PlayRho reference itself.

Fixtures (tests/golden/ref_*.npz) come from tests/golden/make_golden.py, which
runs each scene through the reference library compiled from source.  The oracle
must reproduce them bit for bit: positions, velocities, awake flags, contact
keys, contact features, manifold points and step statistics (with the TOI
phase's statistics for the fixtures that enable it).  Runs without the
reference sources or a GPU.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle
from playrho_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))


def load_scene(z):
    fields = {f.name for f in scenes.Scene.__dataclass_fields__.values()}
    return scenes.Scene(**{f: z[f"scene_{f}"] for f in fields if f"scene_{f}" in z})


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_reproduces_reference(path):
    z = np.load(path)
    double = path.endswith("_f64.npz")
    ow = oracle.OracleWorld(load_scene(z), double=double)
    conf = {k[len("conf_"):]: z[k].item() for k in z.files if k.startswith("conf_")}
    done = 0
    for i, s in enumerate(z["steps"]):
        while done < s:
            st = ow.step(**conf)
            done += 1
        b = ow.bodies()
        np.testing.assert_array_equal(b["pos"], z[f"d{i}_pos"], err_msg=f"positions after {s} steps")
        np.testing.assert_array_equal(b["vel"], z[f"d{i}_vel"], err_msg=f"velocities after {s} steps")
        np.testing.assert_array_equal(b["awake"], z[f"d{i}_awake"], err_msg=f"awake after {s} steps")
        got = [st[k] for k in ("preProxiesCreated", "preContactsDestroyed", "preContactsAdded", "regIslandsFound",
                               "regIslandsSolved", "regContactsAdded", "regBodiesSlept", "regSumPosIters",
                               "regSumVelIters")]
        np.testing.assert_array_equal(got, z[f"d{i}_stats"], err_msg=f"step statistics after {s} steps")
        if f"d{i}_toistats" in z:
            toi = [st[k] for k in oracle.TOI_STATS_INT_FIELDS]
            np.testing.assert_array_equal(toi, z[f"d{i}_toistats"], err_msg=f"TOI statistics after {s} steps")
        if f"d{i}_c_proxy" in z:
            c = ow.contacts()
            np.testing.assert_array_equal(c["proxy"], z[f"d{i}_c_proxy"])
            np.testing.assert_array_equal(c["count"], z[f"d{i}_c_count"])
            np.testing.assert_array_equal(c["type"], z[f"d{i}_c_type"])
            np.testing.assert_array_equal(c["touching"], z[f"d{i}_c_touching"])
            for k in range(len(c["count"])):
                n = int(c["count"][k])
                np.testing.assert_array_equal(c["features"][k][:n], z[f"d{i}_c_features"][k][:n])
                np.testing.assert_array_equal(c["points"][k][:n], z[f"d{i}_c_points"][k][:n])
