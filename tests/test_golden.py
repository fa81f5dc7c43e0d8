"""The committed golden frames (tests/golden, made by make_golden.py).

CPU: the oracle still renders each case's committed frame -- bit-exact when
the scene inputs hash to the recorded digest (same generator output), else
under the parity bars (a platform whose libm rounds exp / sin in the scene
generators differently).  GPU: the CUDA path against the committed frame
under the parity bars of test_gpu_parity.py: first-hit (geomID, primID)
agreement >= 99.9 %, PSNR >= 45 dB linear and sRGB, max |error| <= 1e-3 on
output pixels whose subpixels agree on the first hit (at the 0.999 quantile
and every pixel within 0.3 where AO / soft-shadow sample directions, which
come from sin / cos, may differ in the last bit; GI frames at the 99th
percentile, as the GI parity tests hold them).
"""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

from parity import agree_mask_final, id_agreement, psnr_linear, psnr_srgb

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import golden_cases  # noqa: E402

MANIFEST = json.loads((GOLDEN / "golden.json").read_text())
NAMES = sorted(MANIFEST)


def _load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    return z["color"], z["hit_geom"], z["hit_prim"]


def _bars(color, geom, prim, ref, ss, sampled):
    rc, rg, rp = ref
    agree = id_agreement(geom, prim, rg, rp)
    m = agree_mask_final(geom, prim, rg, rp, ss)
    diff = np.abs(color - rc)[m]
    # GI: the bars of the GI parity tests (|error| <= 1e-3 at the 99th percentile)
    q = 0.99 if sampled == "gi" else 0.999 if sampled else 1.0
    err = float(np.quantile(diff, q)) if diff.size else 0.0
    worst = float(diff.max()) if diff.size else 0.0
    info = dict(agree=agree, err=err, worst=worst, psnr_linear=psnr_linear(color, rc),
                psnr_srgb=psnr_srgb(color, rc))
    assert agree >= 0.999, info
    assert info["psnr_linear"] >= 45.0 and info["psnr_srgb"] >= 45.0, info
    assert err <= 1e-3, info
    if sampled is True:
        assert worst <= 0.3, info


def test_manifest_lists_every_case():
    assert set(MANIFEST) == set(golden_cases.CASES)
    for name in NAMES:
        color, geom, prim = _load(name)
        e = MANIFEST[name]
        ss = e["supersample"]
        assert color.shape == (e["height"], e["width"], 4) and color.dtype == np.float32
        assert geom.shape == prim.shape == (e["height"] * ss, e["width"] * ss)
        assert (geom != 0xFFFFFFFF).any(), name  # every case shows geometry


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name, oracle_lib):
    make, sampled = golden_cases.CASES[name]
    sc, opt = make()
    fr = oracle_lib.render(sc, opt)
    ref = _load(name)
    if golden_cases.digest(sc, opt) == MANIFEST[name]["digest"]:
        assert np.array_equal(fr.color, ref[0])
        assert np.array_equal(fr.hit_geom, ref[1]) and np.array_equal(fr.hit_prim, ref[2])
    else:
        _bars(fr.color, fr.hit_geom, fr.hit_prim, ref, max(1, opt.supersample), sampled)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(name, gpu_ctx):
    make, sampled = golden_cases.CASES[name]
    sc, opt = make()
    b = gpu_ctx.build(sc)
    try:
        g = gpu_ctx.render(b, sc, opt)
    finally:
        b.release()
    _bars(g.color, g.hit_geom, g.hit_prim, _load(name), max(1, opt.supersample), sampled)
