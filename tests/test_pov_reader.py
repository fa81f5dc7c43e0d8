"""The .pov / .inc readers (umbreon_gb300/host/pov/) on the CPU.

* The reference's own reader tests (tests/test_pov_scene_reader.cpp with the
  real CueMol scenes data/test1.pov and data/1ab0_scene1.pov, and
  tests/test_mesh2_reader.cpp), compiled unchanged against this library's
  headers and readers, pass every check.
* tests/cpp/pov_dump.cpp, built once against this library and once against
  the reference's reader sources (src/bench/pov, src/bench/geom), prints the
  same bytes (floats in hex) for every .pov under the reference's data/
  and for seeded synthetic CueMol geometry files covering every construct
  the geometry reader handles.
* Without the reference sources, this library's reader still reads a
  synthetic scene and geometry to their known values.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path("/root/reference")
HOST_INC = ROOT / "umbreon_gb300" / "host" / "include"
LIB = ROOT / "umbreon_gb300" / "lib"
have_ref = (REF / "src" / "bench" / "pov" / "pov_scene_reader.cpp").exists()
needs_ref = pytest.mark.skipif(not have_ref, reason="reference sources absent")


def _ours(tmp_path, src, name):
    from umbreon_gb300 import build
    build.build_ubr()
    build.build_host()
    exe = tmp_path / name
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", str(HOST_INC)] + src + [
        "-L", str(LIB), "-lumbreon_gb300", "-lubr", f"-Wl,-rpath,{LIB}", "-pthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _ref_dump(tmp_path):
    src = REF / "src"
    exe = tmp_path / "pov_dump_ref"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-w", "-I", str(src / "umbreon"), "-I", str(src / "bench")]
    cmd += [str(p) for p in sorted((src / "bench" / "pov").glob("*.cpp")) + sorted((src / "bench" / "geom").glob("*.cpp"))]
    cmd += [str(ROOT / "tests" / "cpp" / "pov_dump.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run(exe, *args):
    r = subprocess.run([str(exe)] + [str(a) for a in args], capture_output=True, text=True, timeout=120)
    return r.returncode, r.stdout


@needs_ref
@pytest.mark.parametrize("name,args", [
    ("test_pov_scene_reader", ["data/test1.pov", "data/1ab0_scene1.pov"]),
    ("test_mesh2_reader", []),
])
def test_reference_reader_tests_pass(tmp_path, name, args):
    exe = _ours(tmp_path, [str(REF / "tests" / f"{name}.cpp"), "-I", str(REF / "tests")], name)
    rc, out = _run(exe, *[REF / a for a in args])
    assert rc == 0, out[-3000:]
    summary = [ln for ln in out.splitlines() if "checks passed" in ln]
    done, total = summary[-1].split("]")[-1].split()[0].split("/")
    assert done == total and int(total) >= 16, summary[-1]


@pytest.fixture(scope="module")
def dumps(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("pov")
    return _ours(tmp, [str(ROOT / "tests" / "cpp" / "pov_dump.cpp")], "pov_dump"), _ref_dump(tmp)


@needs_ref
@pytest.mark.parametrize("pov", sorted(p.name for p in (REF / "data").glob("*.pov")) if have_ref else [])
@pytest.mark.parametrize("opts", [
    ["300", "300"],
    ["640", "360", "_perspective=1", "_light_inten=1.3", "_flash_frac=0.6", "_stereo=1", "_iod=0.05"],
    ["300", "300", "_perspective=0", "_light_inten=1.3", "_flash_frac=0.6", "_amb_frac=0.1", "_radiosity=1"],
])
def test_scene_reader_equals_the_references(dumps, pov, opts):
    ours, ref = dumps
    a = _run(ours, "scene", REF / "data" / pov, *opts)
    b = _run(ref, "scene", REF / "data" / pov, *opts)
    assert a == b


def synthetic_inc(seed):
    """A seeded CueMol-style geometry file: #declare'd vectors and textures,
    one to three mesh2 blocks inside `#if (_show_*)` groups (per-corner or
    per-face texture indices, rgb / rgbt / srgb colours, finishes with named
    metal presets and metallic amounts, a block without normals), spheres
    (one a silhouette joint), raw / open cylinders, edge_line and edge_line2
    calls, a macro definition and a function call in an expression."""
    rng = np.random.default_rng(seed)
    f = lambda x: f"{x:.6g}"
    vec = lambda v: "<" + ", ".join(f(x) for x in v) + ">"
    out = ["#declare _base = <0.2, 0.4, 0.6>;", "#declare _rise = 0.01 * 2;", "#declare _w = sqrt(4);",
           "#macro edge_line(v1, n1, v2, n2, r, w, t, c)", "  cylinder { v1 + r*n1, v2 + r*n2, w open }",
           "#end",
           "#declare _tex_a = texture { pigment { color rgb _base * 0.5 + <0.1, 0, 0> } "
           "finish { ambient 0.3 diffuse 0.6 specular 0.4 roughness 0.01 phong 0.2 phong_size 30 } }",
           "#declare _tex_m = texture { _tex_a finish { F_MetalC metallic 0.5 reflection 0.3 } }"]
    for blk in range(int(rng.integers(1, 4))):
        show = f"_show_{seed}_{blk}"
        nv = int(rng.integers(4, 12))
        verts = rng.uniform(-5, 5, size=(nv, 3)).round(3)
        verts[nv // 2] = verts[0]  # a shared position: one class, maybe two render vertices
        out.append(f"#if ({show})")
        out.append("union { mesh2 {")
        out.append("  vertex_vectors { %d, %s }" % (nv, ", ".join(vec(v) for v in verts)))
        if blk != 1:
            nrm = rng.normal(size=(nv, 3))
            nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
            out.append("  normal_vectors { %d, %s }" % (nv, ", ".join(vec(v) for v in nrm.round(4))))
        kinds = ["rgb", "rgbt", "srgb", "rgbf", "srgbt"]
        nt = int(rng.integers(1, 4))
        texs = []
        for t in range(nt):
            kind = kinds[int(rng.integers(len(kinds)))]
            c = rng.uniform(0, 1, size=4 if "t" in kind or "f" in kind else 3).round(3)
            fin = "" if t else " finish { ambient 0.1 diffuse 0.7 specular %s }" % f(rng.uniform(0, 1))
            texs.append(f"texture {{ pigment {{ color {kind} {vec(c)} }}{fin} }}")
        if blk == 2:
            texs[0] = "texture { _tex_m }"
        out.append("  texture_list { %d, %s }" % (nt, ", ".join(texs)))
        nf = int(rng.integers(2, 8))
        faces = []
        for _ in range(nf):
            idx = rng.choice(nv, 3, replace=False)
            if rng.uniform() < 0.5:
                faces.append(f"{vec(idx)}, {int(rng.integers(nt))}")
            else:
                faces.append(f"{vec(idx)}, " + ", ".join(str(int(rng.integers(nt))) for _ in range(3)))
        out.append("  face_indices { %d, %s }" % (nf, ", ".join(faces)))
        out.append("} }")
        out.append("#end")
    for s in range(int(rng.integers(0, 4))):
        c = rng.uniform(-3, 3, size=3).round(3)
        tex = "_sl_tex" if s == 0 else "_tex_a"
        out.append(f"sphere {{ {vec(c)}, {f(rng.uniform(0.1, 1))} texture {{ {seed}{tex} pigment {{ color rgb "
                   f"{vec(rng.uniform(0, 1, 3).round(3))} }} }} }}")
    out.append("#if (_show_cyl)")
    for s in range(int(rng.integers(0, 3))):
        a, b = rng.uniform(-3, 3, size=(2, 3)).round(3)
        opn = " open" if s % 2 else ""
        out.append(f"cylinder {{ {vec(a)}, {vec(b)}, {f(rng.uniform(0.05, 0.3))}{opn} texture {{ pigment {{ "
                   f"color rgb {vec(rng.uniform(0, 1, 3).round(3))} }} finish {{ F_MetalA }} }} }}")
    a, n1, b, n2 = rng.uniform(-1, 1, size=(4, 3)).round(3)
    out.append(f"edge_line({vec(a)}, {vec(n1)}, {vec(b)}, {vec(n2)}, _rise, 0.05, _tex_a, <0.1, 0.2, 0.3>)")
    out.append(f"edge_line2({vec(a)}, {vec(n1)}, 0.25, {vec(b)}, {vec(n2)}, 0.75, _rise, _w * 0.02, _tex_a, "
               "<0, 0, 0>)")
    out.append("#end")
    return "\n".join(out) + "\n"


@needs_ref
@pytest.mark.parametrize("seed", range(12))
def test_geometry_reader_equals_the_references(dumps, tmp_path, seed):
    ours, ref = dumps
    p = tmp_path / f"synthetic_{seed}.inc"
    p.write_text(synthetic_inc(seed))
    a = _run(ours, "geom", p, "_show_x=1")
    b = _run(ref, "geom", p, "_show_x=1")
    assert a[0] == 0, a[1][-2000:]
    assert a == b


def test_readers_known_values(tmp_path):
    """Without the reference: a small scene and geometry read to the values
    the file states."""
    exe = _ours(tmp_path, [str(ROOT / "tests" / "cpp" / "pov_dump.cpp")], "pov_dump")
    pov = tmp_path / "s.pov"
    pov.write_text("""
#declare _distance = 80;
#declare _zoomy = 12;
global_settings { assumed_gamma 1.8 }
background { color rgb <0.25, 0.5, 1> }
#ifndef (_perspective) #declare _perspective = 0; #end
camera {
#if (_perspective)
  perspective location <0,0,_distance> look_at <0,0,0> angle 30
#else
  orthographic location <0,0,_distance> look_at <0,0,0> up <0,_zoomy,0> right <_zoomy,0,0>
#end
}
SpecLighting(2, _distance, 0.5, 1)
FlashLighting(0.25)
fog { distance 12 color rgb <0.25, 0.5, 1> fog_type 2 up <0,0,1> }
#declare _scene = #include "geom.inc"
""")
    rc, out = _run(exe, "scene", pov, 320, 240)
    assert rc == 0, out
    kv = {ln.split(" ", 1)[0]: ln.split(" ", 1)[1] for ln in out.splitlines()}
    hexf = lambda s: [float.fromhex(x) for x in s.split()]
    assert kv["camera.orthographic"] == "1"
    assert hexf(kv["camera.height"]) == [12.0]
    assert hexf(kv["camera.position"]) == [0.0, 0.0, 80.0]
    assert hexf(kv["background"]) == [0.25, 0.5, 1.0]
    assert hexf(kv["assumedGamma"])[0] == pytest.approx(1.8)
    assert hexf(kv["fog.start"]) == [80.0] and hexf(kv["fog.end"]) == [98.0]
    assert kv["include"] == "geom.inc"
    lights = [ln for ln in out.splitlines() if ln.startswith("light.intensity")]
    assert [hexf(ln.split(" ", 1)[1])[0] for ln in lights] == [0.5, 0.25]
    inc = tmp_path / "g.inc"
    inc.write_text("""
#if (_show_a)
mesh2 { vertex_vectors { 4, <0,0,0>, <1,0,0>, <0,1,0>, <1,1,0> }
        normal_vectors { 4, <0,0,1>, <0,0,1>, <0,0,1>, <0,0,1> }
        texture_list { 1, texture { pigment { color rgbt <1, 0.5, 0, 0.25> } finish { F_MetalB } } }
        face_indices { 2, <0,1,2>, 0, <1,3,2>, 0 } }
#end
sphere { <0,0,1>, 0.5 texture { pigment { color rgb 1 } } }
edge_line2(<0,0,0>, <0,0,1>, 0.2, <1,0,0>, <0,0,1>, 0.6, 0.1, 0.05, t, <0,0,0>)
""")
    rc, out = _run(exe, "geom", inc)
    assert rc == 0, out
    lines = out.splitlines()
    assert lines[0] == "vertices 4 triangles 2 classes 4"
    assert "c 0x1p+0 0x1p-1 0x0p+0 0x1.8p-1" in lines  # rgbt: opacity 1 - 0.25
    assert "tri 0 group 1" in lines and "groupName '_a'" in lines
    assert any(ln.startswith("material ") and " 1 " in ln for ln in lines)  # F_MetalB: metallic
    assert "group 0 open 1 edge 1" in lines
