#!/usr/bin/env python
"""Benchmark: umbreon ray-cast + shade on GB300 through the C-ABI.

A step is one frame of the ball-and-stick workload (20,000 atoms r 0.4 on a
1.5 A random walk + 19,999 capped bonds r 0.2, 2 lights with hard shadows,
16 AO rays at distance 6, 1920x1080 with 2x2 supersampling, linear fog),
rendered with the scene already built in device memory.  `value` is traced
rays (closest-hit + AO/shadow any-hit) per second over the K timed frames;
`e2e` is the same metric through the reference-facing call with HOST
buffers: scene upload + GPU BVH build + render + copy of the frame back.

--impl reference times the reference's CPU path on the host cores.  The
reference itself (Embree 4 + oneTBB) cannot be built on the GPU host, so
this arm runs the CPU restatement of the same path (oracle/, kind "port")
on all host threads; every step renders the whole frame, and rays are
counted as the GPU counts them (closest-hit calls + AO / shadow rays handed
to a traversal).

Multi-GPU: frames are independent, so N GPUs run N replicas of the frame
(weak scaling, no collective on the data path): under torchrun each rank
renders the headline frame on its own GPU; `--gpus N` without torchrun
starts the N ranks itself.  With N > 1 the 64-frame turntable list is also
split into contiguous blocks, one per rank.
"""
from __future__ import annotations

import argparse
import copy
import hashlib
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from umbreon_gb300 import replicas  # noqa: E402

METRIC = "ms/frame & Mrays/s (batched vs per-frame GPU) at >=45 dB PSNR; adjoint ms/iter"
WORKLOAD = "ball_and_stick_20k_1920x1080_ss2_ao16_2lights_shadows_fog"
# --workload: the scene of the headline line (the others are for profiling one workload alone)
WORKLOADS = {
    "ball_and_stick": ("ball_and_stick", WORKLOAD),
    "space_filling": ("space_filling", "space_filling_2k_640x480"),
    "molecular_surface": ("molecular_surface", "molecular_surface_2m_tris_2048_alpha0.5_4layers_ao32_shadows"),
    "differentiable": ("differentiable", "spheres_100k_1024_ao16_enhanced_1light_shadows_fog"),
}


def _workload(args):
    from umbreon_gb300 import scenes
    fn, name = WORKLOADS[args.workload]
    sc, opt = getattr(scenes, fn)()
    return sc, opt, name


def _dist():
    return replicas.env_ranks()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.before = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a while to start: wait (bounded) for its first
            # line, then keep only what it samples inside the timed region
            t0 = time.perf_counter()
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.005)
            self.before = list(self.lines)
            self.lines.clear()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # a region shorter than one sampling period: the sample taken just
        # before it stands in (reported with samples 0)
        lines, inside = (self.lines, True) if self.lines else (self.before[-1:], False)
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm) if inside else 0, "interval_ms": 25}


# the sources that define the trace kernels and their build flags: a DRAM
# traffic figure captured by ncu holds for the kernels these files built
TRAFFIC_SOURCES = ("umbreon_gb300/csrc/render.cu", "umbreon_gb300/csrc/trace.cuh",
                   "umbreon_gb300/csrc/ubr_internal.h", "umbreon_gb300/csrc/gi.cuh", "umbreon_gb300/build.py")


def kernel_digest() -> str:
    h = hashlib.sha256()
    for f in TRAFFIC_SOURCES:
        h.update((ROOT / f).read_bytes())
    return h.hexdigest()[:16]


def _traffic(kernel: str, rays: int):
    """DRAM bytes of one launch of `kernel`: the committed ncu capture's bytes
    per ray times the rays this launch traced, and whether the capture was of
    the kernels built from the current sources."""
    tfile = ROOT / "profiles" / "traffic.json"
    if not tfile.exists():
        return None, None
    d = json.loads(tfile.read_text()).get(kernel)
    if not isinstance(d, dict):
        return None, None
    cap = d["capture"]
    per_ray = cap["dram_bytes"] / cap["rays"]
    info = {"dram_bytes_per_ray": round(per_ray, 3), "captured_rays": cap["rays"],
            "captured_workload": cap["workload"], "current": d.get("kernel_digest") == kernel_digest()}
    return int(round(per_ray * rays)), info


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


L2_POLICY = "flushed (256 MB write) before every timed frame"


def _config(sc, opt, wname, ws):
    """The workload as both arms name it (same keys and values)."""
    return {"workload": wname, "frame": f"{opt.width}x{opt.height} ss{opt.supersample}",
            "spheres": sc.sphere_count(), "cylinders": sc.cylinder_count(), "triangles": sc.triangle_count(),
            "l2": L2_POLICY, "parallelism": f"replicas x{ws}"}


class _CpuFlush:
    """256 MB host write before each timed CPU frame (the CPU arm's cache flush)."""

    def __init__(self):
        import numpy as np
        self.buf = np.empty(256 * 1024 * 1024, np.uint8)
        self.i = 0

    def __call__(self):
        self.i = (self.i + 1) & 255
        self.buf.fill(self.i)


def _cpu_frame(osc, sc, opt, threads, rows=None):
    """One CPU render of the frame (or of a band of hi-res rows): the rays the
    oracle traced (closest-hit calls + AO / shadow rays it handed to a
    traversal, the unit the GPU counts) and the wall time of the call."""
    t0 = time.perf_counter()
    f = osc.render(sc, opt, threads=threads, rows=rows)
    secs = time.perf_counter() - t0
    return {"rays": int(f.stats["rays_primary"] + f.stats["rays_occlusion"]), "secs": secs}


def run_reference(args):
    """The reference's CPU path (its restatement, kind "port") on all host
    threads: every step renders the WHOLE frame of the same workload; the
    value is traced rays over the summed wall time of the K timed frames."""
    ws, rank, local = _dist()
    if rank != 0:
        return
    from oracle import oracle
    sc, opt, wname = _workload(args)
    threads = os.cpu_count() or 1
    osc = oracle.OracleScene(sc)
    flush = _CpuFlush()
    steps = []
    for i in range(args.warmup + args.steps):
        flush()
        r = _cpu_frame(osc, sc, opt, threads)
        if i >= args.warmup:
            steps.append(r)
    secs = sum(s["secs"] for s in steps)
    mrays = sum(s["rays"] for s in steps) / secs / 1e6
    ss = max(1, opt.supersample)
    sample = f"whole frame ({opt.width * ss}x{opt.height * ss} hi-res samples) per step, all host threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(mrays, 3), "unit": "Mrays/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs / len(steps) * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded PCG32 scene generator)",
        "config": _config(sc, opt, wname, ws),
        "rays_per_frame": int(steps[0]["rays"]),
        "cpu_baseline": {"value": round(mrays, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(mrays, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _cpu_baseline(sc, opt, threads, target_s, max_frames=5):
    """The GPU arm's CPU leg: whole frames of the same workload (cache flushed
    before each) until about target_s of CPU work, at least one."""
    from oracle import oracle
    osc = oracle.OracleScene(sc)
    flush = _CpuFlush()
    runs = []
    while not runs or (sum(r["secs"] for r in runs) < target_s and len(runs) < max_frames):
        flush()
        runs.append(_cpu_frame(osc, sc, opt, threads))
    secs = sum(r["secs"] for r in runs)
    ss = max(1, opt.supersample)
    return {"value": round(sum(r["rays"] for r in runs) / secs / 1e6, 3), "unit": "Mrays/s", "cores": threads,
            "kind": "port", "sample": f"{len(runs)} whole frame(s) of {opt.width * ss}x{opt.height * ss} hi-res "
                                      f"samples, all host threads",
            "ms_per_frame": round(secs / len(runs) * 1e3, 1), "rays_per_frame": runs[0]["rays"]}


def _cpu_full_or_band(sc, opt, threads, target_s):
    """CPU restatement on the whole frame when one frame fits in about
    target_s, else on a middle band of hi-res rows sized to about target_s
    (rays counted by the oracle on that band)."""
    from oracle import oracle
    osc = oracle.OracleScene(sc)
    ss = max(1, opt.supersample)
    H = opt.height * ss
    mid = H // 2
    probe_rows = max(2, H // 200)
    r = _cpu_frame(osc, sc, opt, threads, rows=(mid - probe_rows // 2, mid - probe_rows // 2 + probe_rows))
    want = int(min(H, max(2, target_s / max(r["secs"], 1e-6) * probe_rows)))
    if want >= H:
        r = _cpu_frame(osc, sc, opt, threads)
        return {"Mrays_s": round(r["rays"] / r["secs"] / 1e6, 3), "ms_per_frame": round(r["secs"] * 1e3, 1),
                "sample": "whole frame", "cores": threads}
    r0 = max(0, mid - want // 2)
    r = _cpu_frame(osc, sc, opt, threads, rows=(r0, r0 + want))
    return {"Mrays_s": round(r["rays"] / r["secs"] / 1e6, 3),
            "ms_per_frame_est": round(r["secs"] * H / want * 1e3, 1),
            "sample": f"{want} of {H} hi-res rows (middle band)", "cores": threads}


def _device_frames(ctx, built, sc, opt, steps, warmup, flush):
    """Device-resident timing of `steps` frames (outputs in device memory,
    L2 flushed before each frame); returns ms/frame, traced rays/frame and
    one profiled frame's phase split."""
    import ctypes as C
    import torch
    from umbreon_gb300 import abi
    from umbreon_gb300.api import make_render_desc
    rd, keep = make_render_desc(sc, opt)
    col = torch.empty((opt.height, opt.width, 4), dtype=torch.float32, device="cuda")

    def one(flags=0):
        fr = abi.Frame()
        fr.memory = abi.MEMORY_DEVICE
        fr.flags = flags
        fr.color = C.cast(C.c_void_p(col.data_ptr()), abi.f32p)
        ctx._check(ctx._L.ubr_render(ctx.handle, built.handle, C.byref(rd), C.byref(fr), None, None))
        return fr

    for _ in range(warmup):
        one()
    ms, msr, rays = [], [], 0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        fr = one()
        ms.append(fr.total_ms)
        msr.append(fr.render_ms)
        rays += fr.rays_primary + fr.rays_occlusion
    pf = one(abi.FRAME_PROFILE)
    names = ["trace_closest", "surface", "trace_occlusion", "shade", "post"]
    _device_frames.render_ms = sum(msr) / len(msr)
    return (sum(ms) / len(ms), rays / steps, {n: round(v, 3) for n, v in zip(names, pf.phase_ms)},
            pf.layers)


def _adjoint_timing(ctx, built, sc, opt, flush, ms_forward, rays_forward, steps=5, warmup=3):
    """ubr_adjoint with device buffers: dL/dcolour = 2 (frame - 0.5), every
    gradient group returned, interior samples only."""
    import ctypes as C
    import torch
    from umbreon_gb300 import abi
    from umbreon_gb300.api import make_render_desc
    rd, keep = make_render_desc(sc, opt)
    n = sc.sphere_count()
    dcol = torch.full((opt.height, opt.width, 4), 0.1, dtype=torch.float32, device="cuda")
    dcol[..., 3] = 0.0
    gcol = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    gcen = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    grad = torch.empty(n, dtype=torch.float32, device="cuda")

    def one():
        g = abi.Grads()
        g.memory = abi.MEMORY_DEVICE
        g.flags = abi.ADJOINT_INTERIOR_ONLY
        g.sphere_color = C.cast(C.c_void_p(gcol.data_ptr()), abi.f32p)
        g.sphere_center = C.cast(C.c_void_p(gcen.data_ptr()), abi.f32p)
        g.sphere_radius = C.cast(C.c_void_p(grad.data_ptr()), abi.f32p)
        ctx._check(ctx._L.ubr_adjoint(ctx.handle, built.handle, C.byref(rd), C.c_void_p(dcol.data_ptr()),
                                      C.byref(g)))
        return g

    for _ in range(warmup):
        one()
    ms, rays, samples = [], 0, 0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        g = one()
        ms.append(g.adjoint_ms)
        rays += g.rays
        samples = g.samples
    ms_a = sum(ms) / len(ms)
    return {"spheres": n, "frame": f"{opt.width}x{opt.height}", "forward_kernels_ms": round(ms_forward, 3),
            "forward_Mrays_s": round(rays_forward / ms_forward / 1e3, 1), "adjoint_ms": round(ms_a, 3),
            "adjoint_over_forward": round(ms_a / ms_forward, 3), "adjoint_rays": int(rays / steps),
            "timing": "device kernels of one call each (CUDA events), L2 flushed before each call",
            "adjoint_samples": int(samples),
            "gradients": "sphere colour/centre/radius (device arrays) + material, light, ambient, "
                         "background, fog, AO globals"}


def gi_workload(args, flush):
    """GI: (1) the pt1 gather at every pixel (8 spp, one bounce, no denoise)
    on workload 0 with its light shadowed, against the same frame without GI;
    (2) pt1 and pt2 at the reference's defaults on the ball-and-stick frame
    (gather grid = the supersample factor, a-trous denoise of E,
    joint-bilateral upsample, edge patch; pt2 with its Sobol first bounce):
    the GI stages' device ms and rays."""
    import ctypes as C
    import torch
    from umbreon_gb300 import abi, scenes
    from umbreon_gb300.api import Context, make_render_desc
    from umbreon_gb300.autotune import autotune
    out = {}
    sc, opt = scenes.space_filling()
    opt.shadows = True
    knobs = _knobs(args)
    if knobs is None:
        knobs = autotune(sc, opt, pixels=512 * 512)["context"]
    ctx = Context(0, **knobs)
    b = ctx.build(sc)
    ms_d, _, _, _ = _device_frames(ctx, b, sc, opt, 10, 3, flush)
    gi = copy.copy(opt)
    gi.gi, gi.giIntegrator, gi.pt1Denoise, gi.pt1GatherDiv, gi.pt1Spp, gi.giBounces = True, 1, False, 1, 8, 1
    ms_gi, _, _, _ = _device_frames(ctx, b, sc, gi, 10, 3, flush)
    hits = int((ctx.render(b, sc, gi).hit_geom != 0xFFFFFFFF).sum())
    b.release()
    ctx.close()
    g_ms = max(ms_gi - ms_d, 1e-6)
    out["pt1_gi_space_filling_640x480_8spp"] = {
        "ms_per_frame_direct": round(ms_d, 4), "ms_per_frame_gi": round(ms_gi, 4), "gather_ms": round(g_ms, 4),
        "gather_pixels": hits, "gather_Mpaths_s": round(hits * 8 / g_ms / 1e3, 1), "traversal": knobs}
    # the reference's pt1 and pt2 defaults on the headline scene
    sc, opt = scenes.ball_and_stick()
    ctx = Context(0, **(_knobs(args) or {}))
    b = ctx.build(sc)
    ms_d, _, _, _ = _device_frames(ctx, b, sc, opt, 5, 3, flush)
    col = torch.empty((opt.height, opt.width, 4), dtype=torch.float32, device="cuda")
    for integ, key, options, extra in (
            (1, "pt1_gi_defaults_ball_and_stick_1920x1080_ss2",
             "giIntegrator 1, pt1Spp 8, giBounces 1, pt1GatherDiv -1 (= ss 2: 1920x1080 gather grid), "
             "pt1Denoise (a-trous, 5 iterations), upsample, edge patch (spp x4)", {}),
            (2, "pt2_gi_defaults_ball_and_stick_1920x1080_ss2",
             "giIntegrator 2 (the reference's default) with every pt1/pt2 option at its default: the pt1 "
             "pipeline with the blue-noise Owen-scrambled Sobol first bounce; no emitters, no reflective "
             "materials in this scene", {}),
            (2, "pt2_gi_restir_2_rounds_ball_and_stick_1920x1080_ss2",
             "the pt2 defaults with pt2Rounds 2 (ReSTIR spatial resampling, off by default): reservoir "
             "gather (one thread per point) + two spatial rounds, inside gather_ms", {"pt2Rounds": 2})):
        gi = copy.copy(opt)
        gi.gi, gi.giIntegrator = True, integ
        for k, v in extra.items():
            setattr(gi, k, v)
        rd, keep = make_render_desc(sc, gi)
        frames = []
        for i in range(3 + 5):
            flush.zero_()
            torch.cuda.synchronize()
            fr = abi.Frame()
            fr.memory = abi.MEMORY_DEVICE
            fr.color = C.cast(C.c_void_p(col.data_ptr()), abi.f32p)
            ctx._check(ctx._L.ubr_render(ctx.handle, b.handle, C.byref(rd), C.byref(fr), None, None))
            if i >= 3:
                frames.append(fr)
        n = len(frames)
        split = [sum(f.gi_ms[k] for f in frames) / n for k in range(6)]
        gi_ms = sum(split)
        rays = (frames[0].gi_gather_rays + frames[0].gi_nee_rays + frames[0].gi_gbuffer_rays)
        out[key] = {
            "options": options,
            "ms_per_frame_direct": round(ms_d, 3),
            "ms_per_frame_gi": round(sum(f.total_ms for f in frames) / n, 3),
            "gi_ms": round(gi_ms, 3),
            "gi_split_ms": {"gbuffer": round(split[0], 3), "gather": round(split[1], 3),
                            "denoise": round(split[2], 3), "upsample": round(split[3], 3),
                            "edge_patch": round(split[4], 3), "reflection": round(split[5], 3)},
            "gather_rays": int(frames[0].gi_gather_rays), "nee_rays": int(frames[0].gi_nee_rays),
            "gbuffer_rays": int(frames[0].gi_gbuffer_rays), "patched_pixels": int(frames[0].gi_patched_pixels),
            "gi_Mrays_s": round(rays / gi_ms / 1e3, 1)}
    b.release()
    ctx.close()
    return out


def secondary_workloads(args, flush):
    """Workloads 0, 2 and 3 (space filling, molecular surface, batched
    turntable), GPU device-resident, with the CPU restatement beside them."""
    import ctypes as C
    import torch
    from umbreon_gb300 import abi, scenes
    from umbreon_gb300.api import Context, make_render_desc
    from umbreon_gb300.autotune import autotune
    out = {}
    threads = os.cpu_count() or 1

    def tuned(sc, opt):
        """Context with the knobs given on the command line, else autotuned."""
        knobs = _knobs(args)
        if knobs is not None:
            return Context(0, **knobs), knobs
        t = autotune(sc, opt, pixels=512 * 512)
        return Context(0, **t["context"]), t["context"]

    # workload 0
    sc, opt = scenes.space_filling()
    ctx, tn = tuned(sc, opt)
    b = ctx.build(sc)
    ms, rays, ph, layers = _device_frames(ctx, b, sc, opt, 10, 3, flush)
    b.release()
    cpu = _cpu_full_or_band(sc, opt, threads, 2.0) if not args.no_cpu else None
    out["space_filling_2k_640x480"] = {"ms_per_frame": round(ms, 4), "Mrays_s": round(rays / ms / 1e3, 1),
                                       "phase_ms": ph, "cpu": cpu, "traversal": tn}
    ctx.close()
    # workload 2
    t0 = time.perf_counter()
    sc, opt = scenes.molecular_surface()
    gen_s = time.perf_counter() - t0
    mol = (sc, opt)
    ctx, tn = tuned(sc, opt)
    b = ctx.build(sc)
    info = b.info()
    ms, rays, ph, layers = _device_frames(ctx, b, sc, opt, 3, 3, flush)
    b.release()
    cpu = _cpu_full_or_band(sc, opt, threads, 4.0) if not args.no_cpu else None
    mol_knobs = tn
    out["molecular_surface_2048"] = {"triangles": int(info["prim_count"][0]), "spheres": int(info["prim_count"][1]),
                                     "bvh_build_ms": round(info["build_ms"], 1), "generate_s": round(gen_s, 1),
                                     "ms_per_frame": round(ms, 3), "Mrays_s": round(rays / ms / 1e3, 1),
                                     "rays_per_frame": int(rays), "layers": int(layers), "phase_ms": ph,
                                     "cpu": cpu, "traversal": tn}
    ctx.close()
    # adaptive AA (aaMode 1) against the full supersample grid on the
    # ball-and-stick frame and on a molecular surface with mesh AO
    for label, (sc, opt) in (("ball_and_stick_1920x1080_ss2", scenes.ball_and_stick()),
                             ("molecular_surface_1024_ss2", _resized_ss(mol, 1024, 2))):
        ctx, tn = tuned(sc, opt)
        b = ctx.build(sc)
        ms_g, rays_g, _, _ = _device_frames(ctx, b, sc, opt, 5, 3, flush)
        ad = copy.copy(opt)
        ad.aaMode = 1
        ms_a, rays_a, ph_a, _ = _device_frames(ctx, b, sc, ad, 5, 3, flush)
        dbg = copy.copy(ad)
        dbg.aaDebug = True
        flagged = float(ctx.render(b, sc, dbg, want_ids=False).aaMask.mean())
        b.release()
        ctx.close()
        out["adaptive_aa_" + label] = {"grid_ms": round(ms_g, 3), "adaptive_ms": round(ms_a, 3),
                                       "speedup": round(ms_g / ms_a, 2), "flagged_fraction": round(flagged, 4),
                                       "grid_rays": int(rays_g), "adaptive_rays": int(rays_a)}
    # coarse-grid AO (aoResDiv 2: one AO gather per 2x2 block of first hits,
    # interpolated, own rays where the guides reject) against AO rays at
    # every hit, on the molecular surface frame
    sc, opt = mol
    ctx = Context(0, **mol_knobs)
    b = ctx.build(sc)
    ms_i, rays_i, _, _ = _device_frames(ctx, b, sc, opt, 3, 2, flush)
    co = copy.copy(opt)
    co.aoResDiv = 2
    ms_c, rays_c, ph_c, _ = _device_frames(ctx, b, sc, co, 3, 2, flush)
    dbg = copy.copy(co)
    dbg.aoResDebug = True
    patched = float(ctx.render(b, sc, dbg, want_ids=False).aoPatchMask.mean())
    b.release()
    ctx.close()
    out["coarse_ao_molecular_surface_2048"] = {"inline_ms": round(ms_i, 3), "coarse_div2_ms": round(ms_c, 3),
                                               "speedup": round(ms_i / ms_c, 2), "rays_inline": int(rays_i),
                                               "rays_coarse": int(rays_c), "patched_first_hits": round(patched, 4),
                                               "coarse_phase_ms": ph_c}
    # workload 4: forward frame vs adjoint (device buffers, L2 flushed)
    sc, opt = scenes.differentiable()
    ctx, tn = tuned(sc, opt)
    b = ctx.build(sc)
    ms_f, rays_f, ph, _ = _device_frames(ctx, b, sc, opt, 5, 3, flush)
    out["differentiable_100k_1024"] = _adjoint_timing(ctx, b, sc, opt, flush, _device_frames.render_ms, rays_f)
    out["differentiable_100k_1024"]["forward_phase_ms"] = ph
    out["differentiable_100k_1024"]["traversal"] = tn
    b.release()
    ctx.close()
    out["turntable_batch"] = turntable_workload(args, flush)
    out.update(gi_workload(args, flush))
    return out


def turntable_workload(args, flush):
    """Workload 3: the 64-frame turntable list rendered as one batch against
    one frame per call (with and without graph replay), the measured batching
    ceiling, and the same list at 256^2."""
    import ctypes as C
    import torch
    from umbreon_gb300 import abi, scenes
    from umbreon_gb300.api import Context, make_render_desc
    from umbreon_gb300.autotune import autotune
    bases, items = scenes.turntable_batch()
    tune = autotune(items[0][1], items[0][2], pixels=512 * 512)
    res = {"autotune": tune}
    for label, its in (("turntable_64_mixed", items),
                       ("turntable_64_small_256", [(si, sc2, _resized(o, 256)) for si, sc2, o in items])):
        entry = {}
        for mode, graphs in (("batched", True), ("per_frame_graph", True), ("per_frame_no_graph", False)):
            cx = Context(0, graphs=graphs, **(_knobs(args) or tune["context"]))
            built = [cx.build(bs) for bs in bases]
            descs, outs, frames = [], [], []
            for si, sc2, o in its:
                rd, k = make_render_desc(sc2, o)
                descs.append((rd, k))
                t = torch.empty((o.height, o.width, 4), dtype=torch.float32, device="cuda")
                outs.append(t)
                fr = abi.Frame()
                fr.memory = abi.MEMORY_DEVICE
                fr.color = C.cast(C.c_void_p(t.data_ptr()), abi.f32p)
                frames.append(fr)
            arr = (abi.BatchItem * len(its))()
            for i, (si, sc2, o) in enumerate(its):
                arr[i].scene = built[si].handle
                arr[i].desc = C.pointer(descs[i][0])
                arr[i].frame = C.pointer(frames[i])

            def run():
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                if mode == "batched":
                    tot = abi.Frame()
                    cx._check(cx._L.ubr_render_batch(cx.handle, len(its), arr, C.byref(tot)))
                    rays_ = tot.rays_primary + tot.rays_occlusion
                else:
                    rays_ = 0
                    for i, (si, sc2, o) in enumerate(its):
                        cx._check(cx._L.ubr_render(cx.handle, built[si].handle, C.byref(descs[i][0]),
                                                   C.byref(frames[i]), None, None))
                        rays_ += frames[i].rays_primary + frames[i].rays_occlusion
                torch.cuda.synchronize()
                return time.perf_counter() - t1, rays_
            for _ in range(3):
                run()
            runs = [run() for _ in range(5)]
            wall = min(r[0] for r in runs)
            entry[mode] = {"ms_per_batch": round(wall * 1e3, 3), "frames_per_s": round(len(its) / wall, 1),
                           "Mrays_s": round(runs[0][1] / wall / 1e6, 1)}
            if mode == "per_frame_no_graph":
                # the ceiling of batching: every frame's rays at the ray rate
                # the largest frame of its scene reaches alone (a launch that
                # fills the GPU), i.e. no launch gaps, no tails, no idle SMs
                dev = [(frames[i].total_ms, frames[i].rays_primary + frames[i].rays_occlusion, si, o.width)
                       for i, (si, sc2, o) in enumerate(its)]
                rate = {}
                for ms_f, r_f, si, wdt in sorted(dev, key=lambda t: t[3]):
                    rate[si] = r_f / ms_f  # the largest frame of each scene wins
                ideal_ms = sum(r_f / rate[si] for _, r_f, si, _ in dev)
                entry["device_ms_sum_per_frame_path"] = round(sum(d[0] for d in dev), 3)
                entry["ideal_ms_at_full_occupancy"] = round(ideal_ms, 3)
                entry["batching_ceiling_over_per_frame"] = round(wall * 1e3 / ideal_ms, 3)
            for bb in built:
                bb.release()
            cx.close()
        entry["batched_over_per_frame_graph"] = round(entry["batched"]["frames_per_s"] /
                                                      entry["per_frame_graph"]["frames_per_s"], 3)
        entry["batched_over_per_frame_no_graph"] = round(entry["batched"]["frames_per_s"] /
                                                         entry["per_frame_no_graph"]["frames_per_s"], 3)
        entry["pixels"] = int(sum(o.width * o.height for _, _, o in its))
        res[label] = entry
    return res


def _knobs(args):
    """Context tuning fields given on the command line, or None (autotune)."""
    if not (args.builder or args.leaf_max or args.trace_mode or args.collapse or args.sah_scale):
        return None
    return dict(bvh_builder=args.builder, bvh_leaf_max=args.leaf_max, trace_mode=args.trace_mode,
                bvh_collapse=args.collapse, sah_prim_scale=args.sah_scale)


def _resized(opt, res):
    o = copy.copy(opt)
    o.width = o.height = res
    return o


def _resized_ss(scene_opt, res, ss):
    sc, opt = scene_opt
    o = _resized(opt, res)
    o.supersample = ss
    return sc, o


def turntable_partitioned(args, rank, ws, local):
    """The 64-frame turntable list split across ranks (contiguous blocks,
    replicas.partition): each rank builds the scenes its block needs and
    renders its block as one batch; frames/s of the whole job (slowest
    rank's time).  No data crosses ranks."""
    import torch
    from umbreon_gb300 import scenes
    from umbreon_gb300.api import Context
    bases, items = scenes.turntable_batch()
    mine = [items[i] for i in replicas.partition(len(items), rank, ws)]
    ctx = Context(local, **(_knobs(args) or {}))
    built = {si: ctx.build(bases[si]) for si in sorted({it[0] for it in mine})}
    batch = [(built[si], sc, o) for si, sc, o in mine]
    for _ in range(2):
        ctx.render_batch(batch, want_ids=False)

    def step():
        t0 = time.perf_counter()
        ctx.render_batch(batch, want_ids=False)
        torch.cuda.synchronize()
        return len(batch), (time.perf_counter() - t0) * 1e3

    job = replicas.timed_steps(step, 3, sync=torch.cuda.synchronize, device=f"cuda:{local}")
    for b in built.values():
        b.release()
    ctx.close()
    return {"frames_per_s": round(job["units_per_s"], 1), "frames_this_rank": len(mine),
            "ms_per_batch_slowest_rank": round(job["ms_max"] / 3, 3), "timing": "host wall time, 3 batches"}


def run_ours(args):
    import numpy as np
    import torch
    from umbreon_gb300 import abi, scenes
    from umbreon_gb300.api import Context, make_render_desc

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    sc, opt, wname = _workload(args)
    if args.frame:
        opt.width, opt.height = (int(x) for x in args.frame.lower().split("x"))
    if args.ss:
        opt.supersample = args.ss
    # traversal knobs: as given, else what the autotuner picks (downscaled sweep,
    # finalists re-timed on the full frame)
    tune = None
    knobs = _knobs(args)
    if knobs is None:
        from umbreon_gb300.autotune import autotune
        tune = autotune(sc, opt, device=local, pixels=512 * 512)
        knobs = tune["context"]
    ctx = Context(local, **knobs)
    built = ctx.build(sc)
    info = built.info()
    import ctypes as C
    rd, keep = make_render_desc(sc, opt)
    ss = opt.supersample
    W, H = opt.width * ss, opt.height * ss
    dev_color = torch.empty((opt.height, opt.width, 4), dtype=torch.float32, device=f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")  # 256 MB > 129 MB L2

    def frame(flags=0):
        fr = abi.Frame()
        fr.memory = abi.MEMORY_DEVICE
        fr.flags = flags
        fr.color = C.cast(C.c_void_p(dev_color.data_ptr()), abi.f32p)
        st = ctx._L.ubr_render(ctx.handle, built.handle, C.byref(rd), C.byref(fr), None, None)
        if st != abi.UBR_OK:
            ctx._check(st)
        return fr

    for _ in range(args.warmup):
        frame()
    # one counting frame (untimed): algorithmic bytes per ray type
    cf = frame(abi.FRAME_COUNT | abi.FRAME_PROFILE)
    ctr = {"node_bytes": list(cf.node_bytes), "prim_bytes": list(cf.prim_bytes),
           "nodes_visited": list(cf.nodes_visited), "rays": [cf.rays_primary, cf.rays_occlusion]}
    phase = [0.0] * 5
    tally = {"rays": 0, "kernels": 0}

    def step():
        flush.zero_()
        torch.cuda.synchronize()
        fr = frame(abi.FRAME_PROFILE)
        for k in range(5):
            phase[k] += fr.phase_ms[k]
        n = fr.rays_primary + fr.rays_occlusion
        tally["rays"] += n
        tally["kernels"] += fr.kernels
        return n, fr.total_ms

    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        # replicas: the job's time is the slowest rank's, its rays those of all ranks
        job = replicas.timed_steps(step, args.steps, sync=torch.cuda.synchronize, device=f"cuda:{local}")
    wall = time.perf_counter() - wall0
    rays, kernels = tally["rays"], tally["kernels"]
    ms_frame = job["ms_max"] / args.steps
    value = job["units_per_s"] / 1e6

    # roofline of the dominant kernel (per launch = per frame here)
    names = ["trace_closest", "surface", "trace_occlusion", "shade", "post"]
    dom = max(range(5), key=lambda k: phase[k])
    per_launch_ms = phase[dom] / args.steps
    if dom == 2:
        alg = ctr["node_bytes"][1] + ctr["prim_bytes"][1]
    elif dom == 0:
        alg = ctr["node_bytes"][0] + ctr["prim_bytes"][0]
    else:
        alg = None
    peak, peak_kind = _peaks()
    roof = None
    if alg is not None:
        achieved = alg / (per_launch_ms / 1e3) / 1e9
        # DRAM traffic: an ncu capture of a smaller frame, scaled to this
        # launch by the rays it traced; `traffic_source.current` is false when
        # the kernel sources changed after the capture
        traffic, tinfo = _traffic(names[dom], ctr["rays"][1 if dom == 2 else 0])
        roof = {"bound": "hbm", "kernel": f"k_{names[dom]}", "achieved": round(achieved, 1), "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic, "traffic_source": tinfo, "algorithmic_bytes_per_launch": int(alg),
                "launch_ms": round(per_launch_ms, 3)}
        lim = ROOT / "profiles" / "limiter.json"
        if lim.exists():
            # what bounds the kernel in fact (ncu counters of the committed
            # capture): the node bytes come from L1/L2, so the HBM fraction
            # above is a node-fetch delivery rate, not DRAM use
            roof["limiter"] = json.loads(lim.read_text()).get(names[dom])

    # end to end through the C-ABI with host buffers: upload + BVH + render + D2H
    # into a pinned host frame (the caller's buffer; pageable memory works too)
    host_color = torch.zeros((opt.height, opt.width, 4), dtype=torch.float32, pin_memory=True).numpy()
    desc, keepd = sc.to_desc()
    # a one-call render builds the scene every frame: its context is tuned for
    # build + frame (the device-resident number above for the frame alone)
    e2e_knobs = _knobs(args)
    if e2e_knobs is None and not args.no_e2e:
        from umbreon_gb300.autotune import autotune
        e2e_knobs = autotune(sc, opt, device=local, pixels=512 * 512, objective="frame")["context"]
    ectx = Context(local, **e2e_knobs) if not args.no_e2e else ctx
    if not args.no_e2e:  # warm-up: pool growth, graph capture
        hw = C.c_void_p()
        ectx._check(ectx._L.ubr_scene_build(ectx.handle, C.byref(desc), C.byref(hw)))
        frw = abi.Frame()
        frw.memory = abi.MEMORY_HOST
        frw.color = abi.ptr(host_color)
        ectx._check(ectx._L.ubr_render(ectx.handle, hw, C.byref(rd), C.byref(frw), None, None))
        ectx._L.ubr_scene_release(hw)
    h2d = sum(a.nbytes for a in keepd)
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, 5))
    acc = {"build": 0.0, "flat": 0.0, "up": 0.0}

    def e2e_step():
        t0 = time.perf_counter()
        h = C.c_void_p()
        ectx._check(ectx._L.ubr_scene_build(ectx.handle, C.byref(desc), C.byref(h)))
        acc["build"] += time.perf_counter() - t0
        si = abi.SceneInfo()
        ectx._L.ubr_scene_get_info(h, C.byref(si))
        acc["flat"] += si.flatten_ms
        acc["up"] += si.upload_ms
        fr = abi.Frame()
        fr.memory = abi.MEMORY_HOST
        fr.color = abi.ptr(host_color)
        ectx._check(ectx._L.ubr_render(ectx.handle, h, C.byref(rd), C.byref(fr), None, None))
        ectx._L.ubr_scene_release(h)
        return fr.rays_primary + fr.rays_occlusion, (time.perf_counter() - t0) * 1e3

    ejob = replicas.timed_steps(e2e_step, e2e_steps, sync=torch.cuda.synchronize, device=f"cuda:{local}") \
        if e2e_steps else None
    t_build, t_flat, t_up = acc["build"], acc["flat"], acc["up"]
    if ectx is not ctx:
        ectx.close()
    e2e = None if args.no_e2e else {
           "value": round(ejob["units_per_s"] / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(host_color.nbytes), "ms_per_step": round(ejob["ms_max"] / e2e_steps, 2),
           "scene_build_ms_per_step": round(t_build / max(1, e2e_steps) * 1e3, 2),
           "of_which_flatten_ms": round(t_flat / max(1, e2e_steps), 2),
           "of_which_upload_ms": round(t_up / max(1, e2e_steps), 2),
           "steps": e2e_steps, "traversal": e2e_knobs}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = _cpu_baseline(sc, opt, os.cpu_count() or 1, target_s=args.cpu_seconds)

    batch_part = None
    if ws > 1 and not args.no_secondary:
        batch_part = turntable_partitioned(args, rank, ws, local)

    secondary = None
    if rank == 0 and ws == 1 and not args.no_secondary:
        secondary = secondary_workloads(args, flush)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_frame, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded PCG32 scene generator)",
            "config": _config(sc, opt, wname if not (args.frame or args.ss) else wname + "_resized", ws),
            "bvh": {"nodes": info["bvh_nodes"], "primitives_by_kind": info["prim_count"],
                    "traversal": dict(knobs, autotuned=tune["table"] if tune else None,
                                      finalists_full_frame_ms=tune["finalists_full_frame_ms"] if tune else None)},
            "ms_per_frame": round(ms_frame, 3),
            "phase_ms_per_frame": {n: round(v / args.steps, 3) for n, v in zip(names, phase)},
            "rays_per_frame": int(rays / args.steps),
            "wall_s": round(wall, 3),
            "roofline": roof, "counting_frame": ctr, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(kernels), "clocks": clk.summary(),
            "workloads": secondary,
        }
        if batch_part is not None:
            line["turntable_partitioned"] = batch_part
        print(json.dumps(line), flush=True)
    built.release()
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="ball_and_stick", choices=sorted(WORKLOADS),
                    help="scene of the headline line (default: the ball-and-stick benchmark frame)")
    ap.add_argument("--collapse", type=int, default=0, help="8-wide collapse (0 default, 1 greedy, 2 SAH)")
    ap.add_argument("--sah-scale", type=float, default=0.0, help="SAH collapse primitive-cost scale (0 = 1)")
    ap.add_argument("--builder", type=int, default=0, help="BVH builder (0 library default, 1 radix tree, 2 PLOC)")
    ap.add_argument("--no-secondary", action="store_true", help="skip the other workloads (space filling, "
                    "molecular surface, batched turntable)")
    ap.add_argument("--leaf-max", type=int, default=0, help="wide-BVH leaf size 1..3 (0 = library default)")
    ap.add_argument("--trace-mode", type=int, default=0, help="occlusion kernel: 1 per-ray, 2 persistent (0 = default)")
    ap.add_argument("--frame", default=None, help="override the frame size WxH (profiling runs)")
    ap.add_argument("--ss", type=int, default=0, help="override the supersample factor (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # --gpus N outside torchrun: run N ranks (one per GPU) on this node
        sys.exit(replicas.launch(args.gpus, str(Path(__file__).resolve()), sys.argv[1:]))
    ws = _dist()[0]
    if ws != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} but {ws} ranks were started")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
