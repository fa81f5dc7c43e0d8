"""Autotuner for the BVH and traversal knobs of a workload.

Times a representative frame (downscaled to about `pixels` hi-res pixels, so
tuning costs a second or two) for every candidate setting of the context
tuning fields, re-times the best few on the full frame, and returns the
fastest:

* BVH builder: Morton radix tree or PLOC clustering over the same order;
* 8-wide collapse: greedy with a fixed leaf size (1..3 primitives), or the
  SAH-optimal dynamic programme at a few weights of primitive tests against
  node visits (its leaves hold 1..3 primitives as the costs decide);
* occlusion kernel: one thread per ray, persistent warps refilling idle
  lanes, or a resident grid with the top BVH levels in shared memory.

Results depend on the scene's primitive mix and ray lengths, so a caller
tunes once per scene class and creates its context with the result
(`Context(**result["context"])`).
"""
from __future__ import annotations

import copy
import itertools
import math
import time

from .api import Context

# (label, context fields) of the tree candidates
TREES = (
    [(f"greedy_leaf{leaf}", dict(bvh_collapse=1, bvh_leaf_max=leaf)) for leaf in (1, 2, 3)] +
    [(f"sah_x{scale:g}", dict(bvh_collapse=2, sah_prim_scale=scale)) for scale in (1.0, 2.0, 4.0)]
)


def _time(fields, scene, opt, device, repeats, key="total_ms", with_build=False):
    """Best-of-`repeats` frame time of one setting, and (with_build) the best
    scene build wall time: host flattening, upload and device BVH build, which
    a one-call render (`umbreon::render`) pays every frame."""
    ctx = Context(device, **fields)
    try:
        built = ctx.build(scene)
        ctx.render(built, scene, opt, want_ids=False)  # warm-up (graph capture)
        best = min(ctx.render(built, scene, opt, want_ids=False).stats[key] for _ in range(repeats))
        built.release()
        build = 0.0
        if with_build:
            walls = []
            for _ in range(repeats):
                t0 = time.perf_counter()
                b2 = ctx.build(scene)
                walls.append((time.perf_counter() - t0) * 1e3)
                b2.release()
            build = min(walls)
        return best, build
    finally:
        ctx.close()


def autotune(scene, opt, device: int = 0, pixels: int = 256 * 256, repeats: int = 3,
             builders=(1, 2), trees=TREES, trace_modes=(1, 2, 3), finalists: int = 3,
             objective: str = "render"):
    """objective "render": the frame alone (a scene built once, rendered many
    times); "frame": scene build + frame (one render call per scene)."""
    with_build = objective == "frame"
    small = copy.copy(opt)
    ss = max(1, opt.supersample)
    scale = math.sqrt(pixels / float(opt.width * opt.height * ss * ss))
    if scale < 1.0:
        small.width = max(16, int(opt.width * scale))
        small.height = max(16, int(opt.height * scale))
    # the small frame's time scaled to the full frame (plus the build) ranks
    # the candidates
    grow = 1.0 / (scale * scale) if scale < 1.0 else 1.0
    results = {}
    for builder, (tlabel, tfields) in itertools.product(builders, trees):
        for mode in trace_modes:
            fields = dict(tfields, bvh_builder=builder, trace_mode=mode)
            r, bld = _time(fields, scene, small, device, repeats, with_build=with_build)
            results[(builder, tlabel, mode)] = (r * grow + bld, fields)
    ranked = sorted(results.items(), key=lambda kv: kv[1][0])
    final = {}
    if scale < 1.0 and finalists > 1:
        # candidates within a few per cent on the small frame can swap order
        # at full size: re-time the best few on the real frame
        for key, (_, fields) in ranked[:finalists]:
            r, bld = _time(fields, scene, opt, device, repeats, key="render_ms", with_build=with_build)
            final[key] = (r + bld, fields)
        (builder, tlabel, mode), (ms, fields) = min(final.items(), key=lambda kv: kv[1][0])
    else:
        (builder, tlabel, mode), (ms, fields) = ranked[0]
    return {"context": fields, "bvh_builder": builder, "tree": tlabel, "trace_mode": mode, "ms": ms,
            "bvh_leaf_max": fields.get("bvh_leaf_max", 0), "bvh_collapse": fields["bvh_collapse"],
            "sah_prim_scale": fields.get("sah_prim_scale", 0.0),
            "table": {f"builder{b}_{t}_mode{m}": round(v[0], 4) for (b, t, m), v in results.items()},
            "finalists_full_frame_ms": {f"builder{b}_{t}_mode{m}": round(v[0], 4) for (b, t, m), v in final.items()}}
