"""Write the golden fixtures: the CPU oracle's frames of the seeded cases in
golden_cases.py.

    python tests/golden/make_golden.py

For each case: tests/golden/<case>.npz with the output colour (float32 RGBA
at the final size) and the first-hit geomID / primID planes (uint32 at the
supersampled size), and one entry in tests/golden/golden.json with the input
digest, the sizes and the platform that made it.  The frames come from the
oracle; tests/test_ref_pin.py checks that they are bit for bit the frames
the reference's own render path produces (compiled against the oracle's
Embree / oneTBB stand-ins by oracle/build_ref.py), so the GPU tests compare
against the reference's output.
"""
import json
import platform
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import golden_cases  # noqa: E402


def main() -> None:
    from umbreon_gb300 import build
    build.build_oracle()
    from oracle import oracle

    manifest = {}
    for name, (make, sampled) in golden_cases.CASES.items():
        sc, opt = make()
        fr = oracle.render(sc, opt)
        np.savez_compressed(HERE / f"{name}.npz", color=fr.color.astype(np.float32),
                            hit_geom=fr.hit_geom.astype(np.uint32), hit_prim=fr.hit_prim.astype(np.uint32))
        manifest[name] = {
            "digest": golden_cases.digest(sc, opt),
            "width": opt.width,
            "height": opt.height,
            "supersample": max(1, opt.supersample),
            "sampled": sampled,
            "made_on": f"{platform.machine()} {platform.system()}, numpy {np.__version__}",
        }
        print(name, manifest[name]["digest"][:12], fr.color.shape)
    (HERE / "golden.json").write_text(json.dumps(manifest, indent=2) + "\n")


if __name__ == "__main__":
    main()
