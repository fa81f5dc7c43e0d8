"""Image / hit-id comparison metrics shared by the parity tests.

PSNR follows the reference's compareImages (src/bench/image/image_io.cpp:231-238):
mean squared error over sRGB-encoded RGB in [0, 1], 10*log10(1/mse), 99 dB
when mse <= 1e-12.  The linear-HDR variant uses the same formula on the
linear values with the peak taken as max(1, max |reference|).
"""
import numpy as np

INVALID = 0xFFFFFFFF


def srgb_encode(v):
    v = np.clip(np.asarray(v, np.float64), 0.0, 1.0)
    return np.where(v <= 0.0031308, 12.92 * v, 1.055 * np.power(v, 1.0 / 2.4) - 0.055)


def psnr_srgb(a, b):
    d = srgb_encode(a[..., :3]) - srgb_encode(b[..., :3])
    mse = float(np.mean(d * d))
    return 99.0 if mse <= 1e-12 else 10.0 * np.log10(1.0 / mse)


def psnr_linear(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    peak = max(1.0, float(np.max(np.abs(ref))))
    mse = float(np.mean((a - ref) ** 2))
    return 99.0 if mse <= 1e-12 * peak * peak else 10.0 * np.log10(peak * peak / mse)


def id_agreement(ga, pa, gb, pb):
    """Fraction of hi-res pixels whose first-hit (geomID, primID) agree."""
    return float(np.mean((ga == gb) & (pa == pb)))


def agree_mask_final(ga, pa, gb, pb, ss):
    """Output pixels all of whose ss x ss subpixels agree on the first hit."""
    agree = (ga == gb) & (pa == pb)
    H, W = agree.shape
    return agree.reshape(H // ss, ss, W // ss, ss).all(axis=(1, 3))


def interior_mask(g, p, ss):
    """Output pixels whose own subpixels and 3x3 neighbourhood share one hit id
    (excludes silhouettes, where a tie may resolve either way)."""
    key = (g.astype(np.uint64) << np.uint64(32)) | p.astype(np.uint64)
    H, W = key.shape
    k = key.reshape(H // ss, ss, W // ss, ss).transpose(0, 2, 1, 3).reshape(H // ss, W // ss, ss * ss)
    same = (k == k[..., :1]).all(-1)
    c = k[..., 0]
    out = same.copy()
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            sh = np.roll(np.roll(c, dy, 0), dx, 1)
            out &= sh == c
    out[0, :] = out[-1, :] = False
    out[:, 0] = out[:, -1] = False
    return out
