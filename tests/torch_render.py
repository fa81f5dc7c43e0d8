"""Optional torch binding of the differentiable sphere frame, for tests only:
``SphereRender`` is a ``torch.autograd.Function`` whose forward is
``ubr_render`` and whose backward is ``ubr_adjoint`` (device buffers both
ways).  The library itself has no torch dependency."""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np
import torch

from umbreon_gb300 import abi
from umbreon_gb300.api import Context, DistantLight, RenderOptions, Scene, make_render_desc

MATERIAL_FIELDS = abi.MATERIAL_GRAD_FIELDS


def _scene_with(base: Scene, colors, centers, radii, material, light_dir, light_intensity) -> Scene:
    sc = copy.copy(base)
    n = len(colors)
    cr = np.empty((n, 4), np.float32)
    cr[:, :3] = centers
    cr[:, 3] = radii
    col = np.ones((n, 4), np.float32)
    col[:, :3] = colors
    mats = np.array(base.sphere_material, abi.MATERIAL_DTYPE, copy=True)
    for k, name in enumerate(MATERIAL_FIELDS):
        mats[name] = material[k]
    sc.sphere_center_radius, sc.sphere_color, sc.sphere_material = cr, col, mats
    L = base.lights[0]
    sc.lights = [DistantLight(direction=tuple(float(x) for x in light_dir), color=L.color,
                              intensity=float(light_intensity), castsHighlight=L.castsHighlight)] + base.lights[1:]
    return sc


class SphereRender(torch.autograd.Function):
    """image = render(colours (n,3), centres (n,3), radii (n,), material (9,),
    light direction (3,), light intensity ()) for a fixed camera / options."""

    @staticmethod
    def forward(fctx, colors, centers, radii, material, light_dir, light_intensity, ubr: Context, base: Scene,
                opt: RenderOptions):
        sc = _scene_with(base, colors.detach().cpu().numpy(), centers.detach().cpu().numpy(),
                         radii.detach().cpu().numpy(), material.detach().cpu().numpy(),
                         light_dir.detach().cpu().numpy(), light_intensity.detach().cpu().item())
        built = ubr.build(sc)
        rd, keep = make_render_desc(sc, opt)
        out = torch.empty((opt.height, opt.width, 4), dtype=torch.float32, device=colors.device)
        fr = abi.Frame()
        fr.memory = abi.MEMORY_DEVICE
        fr.color = C.cast(C.c_void_p(out.data_ptr()), abi.f32p)
        ubr._check(ubr._L.ubr_render(ubr.handle, built.handle, C.byref(rd), C.byref(fr), None, None))
        fctx.state = (ubr, built, sc, opt, colors.device)
        return out

    @staticmethod
    def backward(fctx, grad_out):
        ubr, built, sc, opt, dev = fctx.state
        rd, keep = make_render_desc(sc, opt)
        n = sc.sphere_count()
        gcol = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        gcen = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        grad = torch.zeros(n, dtype=torch.float32, device=dev)
        go = grad_out.contiguous().to(torch.float32)
        g = abi.Grads()
        g.memory = abi.MEMORY_DEVICE
        g.flags = abi.ADJOINT_INTERIOR_ONLY
        g.sphere_color = C.cast(C.c_void_p(gcol.data_ptr()), abi.f32p)
        g.sphere_center = C.cast(C.c_void_p(gcen.data_ptr()), abi.f32p)
        g.sphere_radius = C.cast(C.c_void_p(grad.data_ptr()), abi.f32p)
        ubr._check(ubr._L.ubr_adjoint(ubr.handle, built.handle, C.byref(rd), C.c_void_p(go.data_ptr()),
                                      C.byref(g)))
        built.release()
        gmat = torch.tensor(list(g.material), dtype=torch.float32, device=dev)
        gdir = torch.tensor(list(g.light_direction[0]), dtype=torch.float32, device=dev)
        gint = torch.tensor(g.light_intensity[0], dtype=torch.float32, device=dev)
        return gcol, gcen, grad, gmat, gdir, gint, None, None, None
