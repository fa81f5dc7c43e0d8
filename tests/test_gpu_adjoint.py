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


def _crop(sc, opt, x0, y0, w, keep):
    """The w x w window at (x0, y0) of an orthographic frame as its own
    frame (same rays up to rounding: the camera moved to the window centre,
    its height scaled), over the spheres `keep`."""
    import copy
    from umbreon_gb300.api import Camera
    c = copy.deepcopy(sc)
    o = copy.deepcopy(opt)
    cam = sc.camera
    D = np.asarray(cam.direction, np.float64)
    D /= np.linalg.norm(D)
    right = np.cross(D, cam.up)
    right /= np.linalg.norm(right)
    up = np.cross(right, D)
    W, H = opt.width, opt.height
    halfH = 0.5 * cam.height
    halfW = halfH * W / H
    pos = (np.asarray(cam.position, np.float64) + right * halfW * (2 * x0 + w - W) / W +
           up * halfH * (H - 2 * y0 - w) / H)
    c.camera = Camera(position=tuple(float(v) for v in pos), direction=cam.direction, up=cam.up,
                      orthographic=True, height=float(cam.height * w / H))
    c.sphere_center_radius = np.ascontiguousarray(sc.sphere_center_radius[keep])
    c.sphere_color = np.ascontiguousarray(sc.sphere_color[keep])
    c.sphere_material = np.ascontiguousarray(np.asarray(sc.sphere_material)[keep])
    o.width = o.height = w
    return c, o


def _window_spheres(sc, lights, opt, x0, y0, w, margin):
    """Spheres that a primary, AO or shadow ray of the window's pixels can
    meet: inside the window's column (inflated by the AO reach), or in the
    column swept back along a light toward the window (shadow rays)."""
    cam = sc.camera
    cr = sc.sphere_center_radius.astype(np.float64)
    W, H = opt.width, opt.height
    halfH = 0.5 * cam.height
    halfW = halfH * W / H
    px, py = cam.position[0], cam.position[1]
    xa, xb = px + halfW * (2 * x0 - W) / W, px + halfW * (2 * (x0 + w) - W) / W
    yb, ya = py + halfH * (1 - 2 * y0 / H), py + halfH * (1 - 2 * (y0 + w) / H)
    reach = cr[:, 3] + opt.aoDistance * 1.3 + margin
    keep = (cr[:, 0] > xa - reach) & (cr[:, 0] < xb + reach) & (cr[:, 1] > ya - reach) & (cr[:, 1] < yb + reach)
    zlo = cr[:, 2].min() - 2.0
    for L in lights:
        d = -np.asarray(L.direction, np.float64)
        d /= np.linalg.norm(d)  # toward the light
        tmax = np.maximum(0.0, (cr[:, 2] - zlo) / max(d[2], 1e-6))
        for f in np.linspace(0.0, 1.0, 64):
            t = tmax * f
            x, y = cr[:, 0] - t * d[0], cr[:, 1] - t * d[1]
            r = cr[:, 3] + margin + tmax / 64 * np.hypot(d[0], d[1])
            keep |= (x > xa - r) & (x < xb + r) & (y > ya - r) & (y < yb + r)
    return np.flatnonzero(keep)


def test_adjoint_benchmark_scene_window(ctx):
    """The benchmarked configuration itself (100,000 spheres, 1024^2, enhanced
    AO 16, one shadowed light, fog): the GPU adjoint of the whole frame with
    the loss on a 32 x 32 window, against FP64 central differences of that
    window (its own frame over the spheres its rays can meet), for every
    global parameter and a dozen spheres."""
    from oracle import fd64
    sc, opt = scenes.differentiable()
    tsc, topt = scenes.differentiable_target(sc, opt)
    x0 = y0 = 496
    w = 32
    keep = _window_spheres(sc, sc.lights + tsc.lights, opt, x0, y0, w, margin=0.2)
    assert 0 < len(keep) < sc.sphere_count()
    csc, copt = _crop(sc, opt, x0, y0, w, keep)
    ctsc, ctopt = _crop(tsc, topt, x0, y0, w, keep)
    seeds = (x0, y0, opt.width)  # the window's pixels seed the full frame's sample streams
    target = fd64.Fd64Frame(ctsc, ctopt, seed_window=seeds).record()
    f = fd64.Fd64Frame(csc, copt, seed_window=seeds)
    img = f.record()
    built = ctx.build(sc)
    try:
        fr = ctx.render(built, sc, opt)
        gid_full = np.where(fr.hit_geom == 0xFFFFFFFF, -1, fr.hit_prim.astype(np.int64))
        gid = gid_full[y0:y0 + w, x0:x0 + w]
        fid = f.primary_ids()
        assert np.mean(np.where(fid < 0, -1, keep[np.maximum(fid, 0)]) == gid) >= 0.999
        # interior samples as the adjoint sees them: the 3x3 neighbourhood in
        # the WHOLE frame (a window-border sample next to another sphere just
        # outside the window is not interior), and interior in the window frame
        wt = (fd64.interior_mask(gid_full)[y0:y0 + w, x0:x0 + w] &
              fd64.interior_mask(fid)).astype(np.float64)
        d_color = np.zeros((opt.height, opt.width, 4), np.float32)
        d_color[y0:y0 + w, x0:x0 + w, :3] = (2.0 * wt[..., None] * (img[..., :3] - target[..., :3])).astype(
            np.float32)
        g = ctx.adjoint(built, sc, opt, d_color, interior_only=True)
    finally:
        built.release()
    rows = _compare(f, g_local(g, keep), GLOBALS, target, wt)
    _check(rows)
    rows = _compare(f, g_local(g, keep), _sphere_params(f, 12, seed=3), target, wt)
    _check(rows, frac_ok=0.95)


def g_local(g, keep):
    """The adjoint's gradients with the per-sphere arrays restricted to the
    window's spheres (indexed as in the window frame)."""
    out = dict(g)
    for k in ("sphere_color", "sphere_center", "sphere_radius"):
        out[k] = np.asarray(g[k])[keep]
    return out
