"""The C++ drop-in layer (umbreon::render over the C-ABI), exercised by C++
test programs compiled against the unchanged public headers."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HOST = ROOT / "umbreon_gb300" / "host"
LIB = ROOT / "umbreon_gb300" / "lib"


def _compile(name: str, tmp_path: Path) -> Path:
    from umbreon_gb300 import build
    build.build_ubr()
    build.build_host()
    exe = tmp_path / name
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(HOST / "include"), "-I", str(ROOT / "include"),
           "-I", str(ROOT / "tests" / "cpp"), str(ROOT / "tests" / "cpp" / f"{name}.cpp"),
           "-L", str(LIB), "-lumbreon_gb300", "-lubr", f"-Wl,-rpath,{LIB}", "-pthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe: Path):
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_host_api_cpu(tmp_path):
    _run(_compile("test_host_cpu", tmp_path))


@pytest.mark.gpu
def test_host_api_render(tmp_path):
    _run(_compile("test_host_render", tmp_path))
