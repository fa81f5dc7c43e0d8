"""The optional torch binding (tests/torch_render.py): autograd through
ubr_render / ubr_adjoint gives the C-ABI's gradients, and gradient descent on
sphere colours and the material fits a target frame."""
import numpy as np
import pytest

from umbreon_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_autograd_binding():
    torch = pytest.importorskip("torch")
    from torch_render import MATERIAL_FIELDS, SphereRender
    from umbreon_gb300.api import Context
    sc, opt = scenes.differentiable(n=300, res=48)
    # target: the same geometry and lights with other colours and finish
    import copy
    tsc = copy.copy(sc)
    rng = np.random.default_rng(7)
    tcol = np.array(sc.sphere_color, np.float32, copy=True)
    tcol[:, :3] = np.clip(tcol[:, :3] + rng.uniform(-0.08, 0.08, (len(tcol), 3)), 0.0, 1.0)
    tsc.sphere_color = tcol
    tm = np.array(sc.sphere_material, copy=True)
    tm["diffuse"] *= 1.15
    tm["specular"] *= 0.8
    tsc.sphere_material = tm
    topt = opt
    ctx = Context(0)
    tb = ctx.build(tsc)
    target = torch.from_numpy(ctx.render(tb, tsc, topt).color).cuda()
    tb.release()
    dev = torch.device("cuda")
    cr = np.asarray(sc.sphere_center_radius, np.float32)
    colors = torch.tensor(np.asarray(sc.sphere_color)[:, :3], device=dev, requires_grad=True)
    centers = torch.tensor(cr[:, :3], device=dev, requires_grad=True)
    radii = torch.tensor(cr[:, 3], device=dev, requires_grad=True)
    m0 = np.asarray(sc.sphere_material)[0]
    material = torch.tensor([float(m0[k]) for k in MATERIAL_FIELDS], device=dev, requires_grad=True)
    L = sc.lights[0]
    ldir = torch.tensor(L.direction, dtype=torch.float32, device=dev, requires_grad=True)
    lint = torch.tensor(L.intensity, dtype=torch.float32, device=dev, requires_grad=True)

    def loss_of():
        img = SphereRender.apply(colors, centers, radii, material, ldir, lint, ctx, sc, opt)
        return ((img[..., :3] - target[..., :3]) ** 2).sum(), img

    loss, img = loss_of()
    loss.backward()
    # the same gradients through the C-ABI directly
    built = ctx.build(sc)
    d = np.zeros((opt.height, opt.width, 4), np.float32)
    d[..., :3] = 2.0 * (img.detach().cpu().numpy()[..., :3] - target.cpu().numpy()[..., :3])
    g = ctx.adjoint(built, sc, opt, d, interior_only=True)
    built.release()
    np.testing.assert_allclose(colors.grad.cpu().numpy(), g["sphere_color"], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(centers.grad.cpu().numpy(), g["sphere_center"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(radii.grad.cpu().numpy(), g["sphere_radius"], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(material.grad.cpu().numpy(), [g[k] for k in MATERIAL_FIELDS], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(ldir.grad.cpu().numpy(), g["light_direction"][0], rtol=1e-4, atol=1e-6)
    # gradient descent on colours and the diffuse / specular weights recovers the target
    opt_t = torch.optim.Adam([colors, material], lr=0.01)
    first = float(loss.detach())
    for _ in range(30):
        opt_t.zero_grad()
        loss, _ = loss_of()
        loss.backward()
        material.grad[[3, 4, 6, 7, 8]] = 0.0  # keep roughness, brilliance, phong size, reflection, emission
        opt_t.step()
        with torch.no_grad():
            colors.clamp_(0.0, 1.0)
    last, _ = loss_of()
    assert float(last.detach()) < 0.2 * first
    ctx.close()
