"""Autotuner for the BVH and traversal knobs of a workload.

Times a representative frame (downscaled to about `pixels` hi-res pixels, so
tuning costs milliseconds) for every combination of the context tuning
fields -- BVH builder (Morton radix tree or PLOC clustering, the latter at
leaf size 1), wide-BVH leaf size (1..3 primitives) and the occlusion kernel
(one thread per ray, or persistent warps refilling idle lanes) -- and returns
the fastest.  Results depend on the scene's primitive mix and ray lengths,
so a caller tunes once per scene class and creates its context with them.
"""
from __future__ import annotations

import copy
import itertools
import math

from .api import Context


def autotune(scene, opt, device: int = 0, pixels: int = 256 * 256, repeats: int = 3,
             leaf_sizes=(1, 2, 3), trace_modes=(1, 2, 3), builders=(1, 2)):
    small = copy.copy(opt)
    ss = max(1, opt.supersample)
    scale = math.sqrt(pixels / float(opt.width * opt.height * ss * ss))
    if scale < 1.0:
        small.width = max(16, int(opt.width * scale))
        small.height = max(16, int(opt.height * scale))
    results = {}
    for builder, leaf, mode in itertools.product(builders, leaf_sizes, trace_modes):
        if builder == 2 and leaf != 1:
            continue  # PLOC trees are built for single-primitive leaves
        ctx = Context(device, bvh_leaf_max=leaf, trace_mode=mode, bvh_builder=builder)
        built = ctx.build(scene)
        try:
            ctx.render(built, scene, small, want_ids=False)  # warm-up (graph capture)
            best = min(ctx.render(built, scene, small, want_ids=False).stats["total_ms"] for _ in range(repeats))
        finally:
            built.release()
            ctx.close()
        results[(builder, leaf, mode)] = best
    (builder, leaf, mode), ms = min(results.items(), key=lambda kv: kv[1])
    return {"bvh_builder": builder, "bvh_leaf_max": leaf, "trace_mode": mode, "ms": ms,
            "table": {f"builder{b}_leaf{l}_mode{m}": round(v, 4) for (b, l, m), v in results.items()}}
