"""prgpu_download_contacts_noalloc against prgpu_download_contacts.

The no-allocation entry point serves callers that must not allocate device
memory once running (allocation-free real-time loops, processes whose device
memory another framework's caching allocator holds).  It stages the gather in a
fixed device array instead of a stream-ordered allocation; its results must be
identical to the allocating entry point's.  This file is collected last so that
a run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from playrho_gb300 import scenes
from playrho_gb300.gpu import GpuBatch, PrgpuError, _ptr

pytestmark = pytest.mark.gpu


def _download(batch, fn_name):
    lib = batch.lib
    fn = getattr(lib, fn_name)
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_void_p] * 8
    n = batch.contact_count()
    cap = max(n, 1)
    out = {
        "proxies": np.zeros((cap, 2), np.uint32), "bodies": np.zeros((cap, 2), np.uint32),
        "flags": np.zeros(cap, np.uint32), "meta": np.zeros((cap, 2), np.int32),
        "head": np.zeros((cap, 4), np.float32), "pts": np.zeros((cap, 8), np.float32),
        "features": np.zeros((cap, 2), np.uint32)}
    nout = ctypes.c_uint32()
    rc = fn(batch.h, cap, ctypes.byref(nout), _ptr(out["proxies"]), _ptr(out["bodies"]), _ptr(out["flags"]),
            _ptr(out["meta"]), _ptr(out["head"]), _ptr(out["pts"]), _ptr(out["features"]))
    batch._check(rc, fn_name)
    return {k: v[: nout.value] for k, v in out.items()}


def _assert_same(a, b):
    assert len(a["proxies"]) == len(b["proxies"])
    for k in a:
        # integer fields and copied floats: the bar is exact equality
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_no_alloc_download_matches_allocating_download(gpu_lib):
    rng = np.random.default_rng(21)
    batch = GpuBatch([scenes.pyramid(rows=10), scenes.pile(300, rng, width=8.0)])
    batch.step_n(90)
    ref = _download(batch, "prgpu_download_contacts")
    assert len(ref["proxies"]) > 100
    # two calls in a row share the same static array
    first = _download(batch, "prgpu_download_contacts_noalloc")
    second = _download(batch, "prgpu_download_contacts_noalloc")
    _assert_same(first, ref)
    _assert_same(second, ref)
    # after more steps the contact set changed; both calls still agree
    batch.step_n(30)
    ref2 = _download(batch, "prgpu_download_contacts")
    _assert_same(_download(batch, "prgpu_download_contacts_noalloc"), ref2)
    _assert_same(_download(batch, "prgpu_download_contacts_noalloc"), ref2)


def test_no_alloc_download_rejects_too_many_contacts(gpu_lib):
    # a batch with more than 65,536 live contacts exceeds the fixed array
    worlds = [scenes.pyramid(rows=20) for _ in range(140)]
    batch = GpuBatch(worlds)
    batch.step_n(20)
    assert batch.contact_count() > 65536
    with pytest.raises(PrgpuError) as e:
        _download(batch, "prgpu_download_contacts_noalloc")
    assert e.value.code == 3  # PRGPU_ECAPACITY
