"""The allocation-free segment-occlusion entry point, through the C-ABI.

ubr_occluded_batch_noalloc serves callers that cannot allocate device memory
at query time (a host with its own strict GPU memory budget, a plugin sandbox
whose host owns all device allocations, a per-frame loop that must not risk
an allocation failure or the synchronisation cudaMalloc/cudaFree can cause).
It must give exactly the answers and status of ubr_occluded_batch --
visibility is a binary answer, so the tolerance is bit equality -- on
consecutive calls that share its one fixed device array, agree with the
oracle's any-hit test on the same segments, accept exactly 524,288 segments
and refuse one more, and leave the device's free memory unchanged.
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


def _noalloc(ctx, built, segs, eps=1e-4):
    n = len(segs)
    out = np.full(n, 7, np.uint8)
    st = ctx._L.ubr_occluded_batch_noalloc(ctx.handle, built.handle, segs.ctypes.data, n, C.c_float(eps),
                                           out.ctypes.data)
    return st, out


def _free_bytes():
    import torch
    return torch.cuda.mem_get_info(0)[0]


def test_noalloc_matches_allocating_entry_and_oracle():
    from oracle import oracle
    sc, _ = scenes.ball_and_stick(n=3000, width=64, height=64, supersample=1)
    osc = oracle.OracleScene(sc)
    ctx = Context(0)
    built = ctx.build(sc)
    try:
        for call, n in enumerate((40000, 123457, MAX_SEGMENTS)):
            segs = _segments(sc, n, seed=100 + call)
            ref = ctx.occluded(built, segs, 1e-4)
            st, out = _noalloc(ctx, built, segs)
            assert st == abi.UBR_OK, ctx._L.ubr_context_last_error(ctx.handle)
            assert np.array_equal(out, ref), f"call {call}: {int((out != ref).sum())} segments differ"
            assert 0 < int(ref.sum()) < n  # both answers occur
            # the same trimmed open segments through the oracle's any-hit test
            # (EmbreeRenderer::occluded plain branch, embree_renderer.cpp:294-315)
            orc = osc.occluded_filtered(segs, 1e-4)
            assert (out == orc).mean() >= 0.9999, f"call {call}: {int((out != orc).sum())} differ from the oracle"
        big = np.zeros((MAX_SEGMENTS + 1, 6), np.float32)
        st, _ = _noalloc(ctx, built, big)
        assert st == abi.UBR_INVALID_ARGUMENT
    finally:
        built.release()
        ctx.close()


def test_noalloc_allocates_nothing_after_its_first_call():
    sc, _ = scenes.ball_and_stick(n=2000, width=64, height=64, supersample=1)
    ctx = Context(0)
    built = ctx.build(sc)
    try:
        segs = _segments(sc, MAX_SEGMENTS, seed=7)
        st, first = _noalloc(ctx, built, segs)  # resolves the array's address
        assert st == abi.UBR_OK
        free0 = _free_bytes()
        for k in range(3):
            st, out = _noalloc(ctx, built, _segments(sc, MAX_SEGMENTS // (k + 1), seed=8 + k))
            assert st == abi.UBR_OK
        st, again = _noalloc(ctx, built, segs)
        assert st == abi.UBR_OK and np.array_equal(again, first)
        assert _free_bytes() == free0
    finally:
        built.release()
        ctx.close()
