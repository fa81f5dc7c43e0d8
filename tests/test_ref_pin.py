"""The oracle pinned on the REFERENCE's own code.

oracle/build_ref.py compiles CueMol/umbreon's render path (src/umbreon,
unmodified, where the sources lie) against the Embree 4 / oneTBB stand-ins
of oracle/shim -- the oracle's BVH and intersectors behind Embree's API --
and the reference's own test programs.  Here (CPU, where the reference
sources exist) that build must pass every check of the reference's render
tests, and the oracle's restatement must reproduce the reference's frames
bit for bit on the golden cases, the benchmark options at reduced size, and
pt1 / pt2 GI at their defaults and with every pt2 feature.  Skipped where
the reference sources are absent (the GPU host).
"""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path("/root/reference")
sys.path.insert(0, str(ROOT / "tests" / "golden"))

pytestmark = pytest.mark.skipif(not (REF / "src" / "umbreon" / "umbreon.cpp").exists(),
                                reason="reference sources absent")

REF_TESTS = ["test_render_shading", "test_render_transparency", "test_render_shadows_gi", "test_render_ao",
             "test_fog", "test_image_ops", "test_clip_planes", "test_mesh_indexed", "test_adaptive_aa",
             "test_ao_coarse", "test_principled", "test_math", "test_render_async", "test_pt1_gather",
             "test_pt1_upsample", "test_pt1_render", "test_pt1_embree", "test_pt2_render"]


@pytest.fixture(scope="module")
def ref_build():
    lib = ROOT / "oracle" / "_ref" / "libumbreon_ref.so"
    srcs = [ROOT / "oracle" / "shim" / "rtcore_shim.cpp", ROOT / "oracle" / "ref" / "ref_driver.cpp",
            ROOT / "oracle" / "src" / "oracle_geom.hpp"]
    stale = not lib.exists() or any(p.stat().st_mtime > lib.stat().st_mtime for p in srcs)
    if stale:
        r = subprocess.run([sys.executable, str(ROOT / "oracle" / "build_ref.py")], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    from oracle import ref
    assert ref.available()
    return ref


@pytest.mark.parametrize("name", REF_TESTS)
def test_reference_tests_pass_on_the_oracle_substrate(ref_build, name):
    exe = ROOT / "oracle" / "_ref" / name
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, "\n".join((r.stdout + r.stderr).splitlines()[-30:])
    summary = [ln for ln in r.stdout.splitlines() if "checks passed" in ln]
    assert summary, r.stdout[-2000:]
    done, total = summary[-1].split("]")[-1].split()[0].split("/")
    assert done == total, summary[-1]


def _cases():
    from golden_cases import CASES
    out = [(name, fn) for name, (fn, _) in CASES.items()]
    from umbreon_gb300 import scenes

    def headline_480():
        return scenes.ball_and_stick(width=480, height=270)

    def gi(integrator, ss, **kw):
        def make():
            sc, opt = scenes.ball_and_stick(n=600, width=64, height=48, supersample=ss, ao_samples=4)
            opt.gi, opt.giIntegrator, opt.pt1Spp = True, integrator, 4
            for k, v in kw.items():
                setattr(opt, k, v)
            return sc, opt
        return make

    def pt2_mixed(ss, mesh=False, **kw):
        def make():
            sys.path.insert(0, str(ROOT / "tests"))
            from test_gpu_pt1 import _pt2_materials
            if mesh:
                sc, opt = scenes.molecular_surface(n_atoms=300, box=14.0, n_spheres=60, width=64, height=64,
                                                   ao_samples=4, layers=2)
            else:
                sc, opt = scenes.ball_and_stick(n=600, width=64, height=48, supersample=ss, ao_samples=4)
            _pt2_materials(sc, mesh=mesh)
            opt.gi, opt.giIntegrator, opt.pt1Spp, opt.pt2GlossySpp = True, 2, 4, 4
            for k, v in kw.items():
                setattr(opt, k, v)
            return sc, opt
        return make

    out += [("ball_and_stick_480x270_ss2_headline_options", headline_480),
            ("pt1_defaults_ss2", gi(1, 2)), ("pt1_full_grid_no_denoise", gi(1, 1, pt1GatherDiv=1, pt1Denoise=False)),
            ("pt1_grid3_three_bounces", gi(1, 1, pt1GatherDiv=3, giBounces=3, pt1Ld=False)),
            ("pt2_defaults_ss2", gi(2, 2)), ("pt2_sobol_pattern", gi(2, 1, pt2Pattern=0)),
            ("pt2_mixed_materials_ss2", pt2_mixed(2)), ("pt2_mixed_materials_adaptive", pt2_mixed(1, pt2Adaptive=True)),
            ("pt2_emissive_mesh", pt2_mixed(1, mesh=True)),
            ("pt2_restir_two_rounds_ss2", gi(2, 2, pt2Rounds=2)),
            ("pt2_restir_unbiased_full_grid", gi(2, 1, pt2Rounds=1, pt1GatherDiv=1, pt2Unbiased=True)),
            ("pt2_restir_three_rounds_clamped", gi(2, 1, pt2Rounds=3, pt2Radius=6.0, pt2WClamp=4.0, pt2MCap=20.0,
                                                   pt2Adaptive=True, pt1Spp=6)),
            ("pt2_restir_emissive_mesh", pt2_mixed(1, mesh=True, pt2Rounds=2, pt2Unbiased=True))]
    return out


@pytest.mark.parametrize("name,make", _cases(), ids=[c[0] for c in _cases()])
def test_restatement_equals_the_reference_bit_for_bit(ref_build, oracle_lib, name, make):
    sc, opt = make()
    o = oracle_lib.render(sc, opt)
    color, depth, vz, _ = ref_build.render(sc, opt)
    assert np.array_equal(o.color, color), float(np.abs(o.color - color).max())
    assert np.array_equal(o.depth, depth)


def test_committed_golden_frames_are_the_references(ref_build):
    """tests/golden's committed frames (the GPU tests' fixtures) are exactly
    what the reference's own code renders for those inputs."""
    import json
    import golden_cases
    manifest = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())
    checked = 0
    for name, (make, _) in golden_cases.CASES.items():
        sc, opt = make()
        if golden_cases.digest(sc, opt) != manifest[name]["digest"]:
            continue  # this platform's scene generator differs: the fixture is not for these inputs
        color, _, _, _ = ref_build.render(sc, opt)
        committed = np.load(ROOT / "tests" / "golden" / f"{name}.npz")["color"]
        assert np.array_equal(color, committed), name
        checked += 1
    assert checked > 0
