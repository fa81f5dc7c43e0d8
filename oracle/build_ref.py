#!/usr/bin/env python
"""Build the REFERENCE's own render path as a CPU checker -- TEST INFRASTRUCTURE.

Compiles CueMol/umbreon's library sources (src/umbreon, the list of its
CMakeLists.txt `umbreon` target) unmodified, where they lie, against the
Embree 4 / oneTBB stand-ins in oracle/shim (the oracle's own BVH and
intersectors behind Embree's API names), plus oracle/ref/ref_driver.cpp,
into oracle/_ref/libumbreon_ref.so; and the reference's own test programs
(tests/*.cpp) into oracle/_ref/.  Nothing is copied out of the reference.
Usable only where the reference sources exist; the outputs are x86 / Arm
binaries of the machine that built them and are not committed.

    python oracle/build_ref.py [--reference DIR] [--jobs N]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_ref"
DEFAULT_REF = Path("/root/reference")

# the reference's `umbreon` library sources (CMakeLists.txt:118-141)
LIB_SOURCES = [
    "render/embree_renderer.cpp", "render/scene_build.cpp", "render/curve_build.cpp", "render/pipeline.cpp",
    "render/render_progress.cpp", "experimental/irradiance_cache/denoise_atrous.cpp",
    "integrator/pt1/pt1_denoise.cpp", "postprocess/fog.cpp", "postprocess/image_ops.cpp",
    "edges/stroke_edges.cpp", "edges/stroke_render.cpp", "edges/screen_edge_classify.cpp",
    "edges/screen_edge_trace.cpp", "edges/screen_edge_prune.cpp", "edges/screen_edge_geometry.cpp",
    "edges/screen_vector_edges.cpp", "edges/mesh_feature_edges.cpp", "edges/screen_projection.cpp",
    "edges/object_space_edges.cpp", "edges/edge_mesh_bvh.cpp", "edges/analytic_silhouette.cpp",
    "umbreon.cpp", "log.cpp",
]
# the reference's tests of the render path (tests/*.cpp, each its own main)
TESTS = [
    "test_render_shading", "test_render_transparency", "test_render_shadows_gi", "test_render_ao", "test_fog",
    "test_image_ops", "test_clip_planes", "test_mesh_indexed", "test_adaptive_aa", "test_ao_coarse",
    "test_principled", "test_math", "test_render_async", "test_pt1_gather", "test_pt1_upsample",
    "test_pt1_render", "test_pt1_embree", "test_pt2_render",
]
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off", "-w"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, r.stdout + r.stderr


def build(reference: Path, jobs: int) -> dict:
    src = reference / "src" / "umbreon"
    inc = ["-I", str(src), "-I", str(HERE / "shim"), "-I", str(HERE / "src"), "-I", str(ROOT / "include")]
    objdir = OUT / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    units = [(src / s, objdir / (s.replace("/", "_") + ".o")) for s in LIB_SOURCES]
    units += [(HERE / "shim" / "rtcore_shim.cpp", objdir / "rtcore_shim.o"),
              (HERE / "ref" / "ref_driver.cpp", objdir / "ref_driver.o")]
    report = {"library": None, "tests": {}}
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(_run, ["g++"] + FLAGS + inc + ["-c", str(s), "-o", str(o)]): s for s, o in units}
        errors = [(str(futs[f]), f.result()[1]) for f in futs if f.result()[0] != 0]
    if errors:
        report["library"] = {"ok": False, "errors": errors}
        return report
    lib = OUT / "libumbreon_ref.so"
    rc, log = _run(["g++", "-shared", "-pthread", "-o", str(lib)] + [str(o) for _, o in units])
    report["library"] = {"ok": rc == 0, "path": str(lib), "log": log[-2000:]}
    if rc != 0:
        return report
    tinc = inc + ["-I", str(reference / "tests")]

    def one(name):
        exe = OUT / name
        return name, _run(["g++"] + FLAGS + tinc + [str(reference / "tests" / (name + ".cpp")), "-o", str(exe),
                                                    str(lib), f"-Wl,-rpath,{OUT}"])

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for name, (rc, log) in ex.map(one, TESTS):
            report["tests"][name] = {"built": rc == 0, "log": log[-1500:] if rc else ""}
    return report


def build_if_stale(reference: Path = DEFAULT_REF, jobs: int = os.cpu_count() or 4, verbose: bool = False) -> bool:
    """Build when the reference sources exist and an output is missing or
    older than the stand-ins, the driver or this recipe.  Returns whether the
    checker is available afterwards."""
    if not (reference / "src" / "umbreon" / "umbreon.cpp").exists():
        return False
    outs = [OUT / "libumbreon_ref.so"] + [OUT / t for t in TESTS]
    deps = [Path(__file__)] + sorted((HERE / "shim").rglob("*")) + sorted((HERE / "ref").glob("*")) + sorted(
        (HERE / "src").glob("*.hpp"))
    deps = [d for d in deps if d.is_file()]
    newest = max(d.stat().st_mtime for d in deps)
    if all(o.exists() and o.stat().st_mtime >= newest for o in outs):
        return True
    rep = build(reference, jobs)
    ok = bool(rep["library"] and rep["library"]["ok"]) and all(t["built"] for t in rep["tests"].values())
    if verbose:
        print(("built " if ok else "FAILED to build ") + str(OUT / "libumbreon_ref.so"))
    return ok


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(DEFAULT_REF))
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    ref = Path(a.reference)
    if not (ref / "src" / "umbreon" / "umbreon.cpp").exists():
        print(f"reference sources not found under {ref}; nothing built")
        return 0
    rep = build(ref, a.jobs)
    lib = rep["library"]
    if not lib["ok"]:
        for f, e in lib.get("errors", [])[:5]:
            print("FAILED", f, "\n", e[-3000:])
        return 1
    for n, t in rep["tests"].items():
        print(("built " if t["built"] else "FAILED ") + n + ("" if t["built"] else "\n" + t["log"]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
