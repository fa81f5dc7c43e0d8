"""The allocation-free segment-occlusion entry point, through the C-ABI.

ubr_occluded_batch_noalloc serves callers that cannot allocate device memory
at query time (a host with its own strict GPU memory budget, a plugin sandbox
whose host owns all device allocations, a per-frame loop that must not risk
an allocation failure or the synchronisation cudaMalloc/cudaFree can cause).
It must give exactly the answers of ubr_occluded_batch -- visibility is a
binary answer, so the tolerance is bit equality -- on consecutive calls that
share its one fixed device array, and refuse more than 524,288 segments.
This file is collected last so a failure here leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest

from umbreon_gb300 import abi, scenes
from umbreon_gb300.api import Context

pytestmark = pytest.mark.gpu

MAX_SEGMENTS = 1 << 19


def _segments(sc, n, seed):
    rng = np.random.default_rng(seed)
    pos = sc.sphere_center_radius[:, :3]
    lo, hi = pos.min(0) - 2.0, pos.max(0) + 2.0
    a = rng.uniform(lo, hi, size=(n, 3))
    b = a + rng.normal(scale=4.0, size=(n, 3))
    return np.ascontiguousarray(np.concatenate([a, b], 1).astype(np.float32))


def test_noalloc_matches_allocating_entry():
    sc, _ = scenes.ball_and_stick(n=3000, width=64, height=64, supersample=1)
    ctx = Context(0)
    built = ctx.build(sc)
    L = ctx._L
    try:
        for call, n in enumerate((40000, 123457)):
            segs = _segments(sc, n, seed=100 + call)
            ref = ctx.occluded(built, segs, 1e-4)
            out = np.full(n, 7, np.uint8)
            st = L.ubr_occluded_batch_noalloc(ctx.handle, built.handle, segs.ctypes.data, n,
                                              C.c_float(1e-4), out.ctypes.data)
            assert st == abi.UBR_OK, L.ubr_context_last_error(ctx.handle)
            assert np.array_equal(out, ref), f"call {call}: {int((out != ref).sum())} segments differ"
            assert 0 < int(ref.sum()) < n  # both answers occur
        big = np.zeros((MAX_SEGMENTS + 1, 6), np.float32)
        res = np.zeros(MAX_SEGMENTS + 1, np.uint8)
        st = L.ubr_occluded_batch_noalloc(ctx.handle, built.handle, big.ctypes.data, MAX_SEGMENTS + 1,
                                          C.c_float(1e-4), res.ctypes.data)
        assert st == abi.UBR_INVALID_ARGUMENT
    finally:
        built.release()
        ctx.close()
