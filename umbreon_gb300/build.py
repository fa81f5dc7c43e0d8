"""Build the native parts in-tree.

* ``umbreon_gb300/lib/libubr.so``: the CUDA library behind ``include/ubr.h``
  (sm_103a only), compiled by nvcc translation unit by translation unit, in
  parallel, then linked with the static CUDA runtime.
* ``umbreon_gb300/lib/libumbreon_gb300.so``: the C++ drop-in host layer
  (``umbreon::render`` and friends) over the C-ABI.
* ``oracle/liboracle.so``: the CPU checker used by the tests and the bench's CPU
  baseline (test infrastructure, built here because ``build()`` builds it).

Host code is compiled with ``-ffp-contract=off`` so float results do not
depend on whether the host compiler fuses multiply-adds (x86 vs. aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "umbreon_gb300"
CSRC = PKG / "csrc"
HOST = PKG / "host"
LIB = PKG / "lib"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["api.cu", "scene_build.cu", "render.cu", "gi.cu", "adjoint.cu"]
HOST_SOURCES = ["umbreon.cpp", "pov/sdl.cpp", "pov/pov_scene_reader.cpp", "pov/mesh2_reader.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libubr")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def build_ubr(verbose: bool = False) -> Path:
    """Compile libubr.so (the CUDA side of the C-ABI)."""
    LIB.mkdir(exist_ok=True)
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
        "-I", str(INCLUDE), "-I", str(CSRC),
    ]
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = objdir / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs + [Path(__file__)]):
            jobs.append([nvcc] + common + ["-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    out = LIB / "libubr.so"
    if jobs or _stale(out, objs):
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-Xlinker", "--no-undefined", "-o", str(out)]
             + [str(o) for o in objs])
    if verbose:
        print("built", out)
    return out


def build_host(verbose: bool = False) -> Path:
    """Compile the C++ drop-in layer (umbreon::render over ubr_*)."""
    LIB.mkdir(exist_ok=True)
    out = LIB / "libumbreon_gb300.so"
    srcs = [HOST / s for s in HOST_SOURCES]
    hdrs = sorted((HOST / "include").rglob("*.hpp")) + sorted((HOST / "pov").glob("*.hpp")) + sorted(INCLUDE.glob("*.h"))
    ubr = LIB / "libubr.so"
    if _stale(out, srcs + hdrs + [ubr]):
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
               "-I", str(HOST / "include"), "-I", str(INCLUDE)] + [str(s) for s in srcs] + [
               "-L", str(LIB), "-lubr", "-Wl,-rpath,$ORIGIN", "-o", str(out)]
        _run(cmd)
    if verbose:
        print("built", out)
    return out


def build_oracle(verbose: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure)."""
    out = ORACLE / "liboracle.so"
    srcs = [ORACLE / "src" / "oracle_render.cpp", ORACLE / "src" / "oracle_fd64.cpp"]
    deps = srcs + sorted((ORACLE / "src").glob("*.hpp")) + sorted(INCLUDE.glob("*.h"))
    if _stale(out, deps):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
              "-I", str(INCLUDE)] + [str(s) for s in srcs] + ["-o", str(out)])
    if verbose:
        print("built", out)
    return out


def build_all(verbose: bool = False) -> None:
    build_oracle(verbose)
    build_ubr(verbose)
    if (HOST / "umbreon.cpp").exists():
        build_host(verbose)
    # the reference's own render path as a CPU checker, only where its
    # sources exist (oracle/build_ref.py)
    sys.path.insert(0, str(ROOT))
    from oracle import build_ref
    build_ref.build_if_stale(verbose=verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
