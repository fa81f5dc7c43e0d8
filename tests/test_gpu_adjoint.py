"""ubr_adjoint against FP64 central finite differences (h = 1e-4) of the
float64 restatement with visibility held fixed (oracle/fd64.py), on a small
instance of the differentiable workload (spheres, enhanced AO with linear
falloff, one shadowed light, fog): relative gradient error <= 1e-3."""
import numpy as np
import pytest

from umbreon_gb300 import scenes

pytestmark = pytest.mark.gpu

H = 1e-4
REL = 1e-3

GLOBALS = ([(n, ()) for n in ("ambient", "diffuse", "specular", "roughness", "phong", "phong_size", "emission")] +
           [("light_direction", (0, k)) for k in range(3)] + [("light_intensity", (0,))] +
           [("light_color", (0, k)) for k in range(3)] + [("ambient_color", (k,)) for k in range(3)] +
           [("background", (k,)) for k in range(3)] + [("fog_start", ()), ("fog_end", ())] +
           [("fog_color", (k,)) for k in range(3)] + [("ao_distance", ()), ("ao_intensity", ()),
                                                      ("specular_scale", ())])


def _adj_value(g, name, idx):
    v = g[name]
    if isinstance(v, float):
        return v
    return float(np.asarray(v)[idx])


def _setup(n, res, interior, **kw):
    from oracle import fd64
    sc, opt = scenes.differentiable(n=n, res=res)
    for k, v in kw.items():
        setattr(opt, k, v)
    tsc, topt = scenes.differentiable_target(sc, opt)
    target = fd64.Fd64Frame(tsc, topt).record()
    f = fd64.Fd64Frame(sc, opt)
    img = f.record()
    w = fd64.interior_mask(f.primary_ids()).astype(np.float64) if interior else np.ones(img.shape[:2])
    d_color = np.zeros(img.shape, np.float32)
    d_color[..., :3] = (2.0 * w[..., None] * (img[..., :3] - target[..., :3])).astype(np.float32)
    return sc, opt, f, img, target, w, d_color


def _sphere_params(f, count, seed=0):
    ids = f.primary_ids()
    cov = np.bincount(ids[ids >= 0], minlength=len(f.sph))
    top = list(np.argsort(-cov)[:count // 2])
    rng = np.random.default_rng(seed)
    seen = np.flatnonzero(cov > 0)
    top += list(rng.choice(seen, size=min(count - len(top), len(seen)), replace=False))
    out = []
    for k in dict.fromkeys(int(x) for x in top):
        out += [("sphere_color", (k, c)) for c in range(3)]
        out += [("sphere_center", (k, c)) for c in range(3)]
        out.append(("sphere_radius", (k,)))
    return out


def _compare(f, g, params, target, w):
    rows = []
    for name, idx in params:
        fd = f.fd(name, idx, target, w, h=H)
        rows.append((name, idx, _adj_value(g, name, idx), fd))
    return rows


def _check(rows, frac_ok=1.0):
    """Each gradient within REL of its finite difference; entries whose FD is
    tiny against the largest of their group (cancellation) are held to REL of
    1 % of that largest value."""
    by = {}
    for name, idx, a, fd in rows:
        by.setdefault(name, []).append((idx, a, fd))
    bad = []
    total = 0
    for name, items in by.items():
        scale = max(abs(fd) for _, _, fd in items)
        for idx, a, fd in items:
            total += 1
            den = max(abs(fd), 1e-2 * scale, 1e-12)
            if abs(a - fd) / den > REL:
                bad.append((name, idx, a, fd, abs(a - fd) / den))
    assert len(bad) <= (1.0 - frac_ok) * total, bad[:10]
    return bad


@pytest.fixture(scope="module")
def ctx():
    from umbreon_gb300.api import Context
    c = Context(0)
    yield c
    c.close()


def test_adjoint_interior_matches_fp64_fd(ctx):
    sc, opt, f, img, target, w, d_color = _setup(300, 48, interior=True)
    built = ctx.build(sc)
    # the forward frame on the GPU is the float64 frame to float rounding
    fr = ctx.render(built, sc, opt)
    gid = np.where(fr.hit_geom == 0xFFFFFFFF, -1, fr.hit_prim.astype(np.int64))
    agree = gid == f.primary_ids()
    assert agree.mean() >= 0.999
    assert np.abs(fr.color[..., :3] - img[..., :3])[agree].max() < 1e-4
    g = ctx.adjoint(built, sc, opt, d_color, interior_only=True)
    # interior samples with a nonzero colour gradient (background matches its target exactly)
    assert 0.95 * w.sum() <= g["stats"]["samples"] <= w.sum()
    rows = _compare(f, g, GLOBALS, target, w)
    _check(rows)
    rows = _compare(f, g, _sphere_params(f, 24), target, w)
    _check(rows, frac_ok=0.98)
    a = np.array([r[2] for r in rows])
    b = np.array([r[3] for r in rows])
    assert np.linalg.norm(a - b) <= REL * np.linalg.norm(b)
    built.release()


def test_adjoint_all_pixels_matches_fp64_fd(ctx):
    """Every pixel, silhouettes included, for the shading, light, fog, AO and
    colour parameters.  (Geometry gradients are held to the bar on interior
    samples only: where a ray grazes a sphere dt/dc grows as 1 / cos of the
    grazing angle, so neither float nor a finite step resolves it.)"""
    sc, opt, f, img, target, w, d_color = _setup(200, 40, interior=False)
    built = ctx.build(sc)
    g = ctx.adjoint(built, sc, opt, d_color, interior_only=False)
    assert g["stats"]["samples"] >= 0.95 * w.size
    colours = [p for p in _sphere_params(f, 12, seed=1) if p[0] == "sphere_color"]
    rows = _compare(f, g, GLOBALS + colours, target, w)
    _check(rows)
    built.release()


def test_adjoint_gamma_supersample_multiscale(ctx):
    """Box downsample, assumed gamma, multi-scale AO and low-discrepancy
    samples in the chain."""
    from oracle import fd64
    sc, opt = scenes.differentiable(n=200, res=24)
    opt.supersample = 2
    opt.aoMultiScale = True
    opt.aoLowDiscrepancy = True
    sc.assumedGamma = 1.8
    tsc, topt = scenes.differentiable_target(sc, opt)
    target = fd64.Fd64Frame(tsc, topt).record()
    f = fd64.Fd64Frame(sc, opt)
    img = f.record()
    # output pixels whose every sub-sample is interior: the loss sees only
    # them, so the samples the interior test drops carry no gradient
    inner = fd64.interior_mask(f.primary_ids())
    w = inner.reshape(opt.height, 2, opt.width, 2).all(axis=(1, 3)).astype(np.float64)
    d_color = np.zeros(img.shape, np.float32)
    d_color[..., :3] = (2.0 * w[..., None] * (img[..., :3] - target[..., :3])).astype(np.float32)
    built = ctx.build(sc)
    g = ctx.adjoint(built, sc, opt, d_color, interior_only=True)
    rows = _compare(f, g, GLOBALS + _sphere_params(f, 8, seed=2), target, w)
    _check(rows, frac_ok=0.98)
    built.release()


def test_adjoint_rejects_unsupported(ctx):
    from umbreon_gb300 import abi
    sc, opt = scenes.ball_and_stick(n=50, width=32, height=32, supersample=1, ao_samples=0)
    built = ctx.build(sc)
    with pytest.raises(abi.UbrError):
        ctx.adjoint(built, sc, opt, np.zeros((32, 32, 4), np.float32))
    built.release()
