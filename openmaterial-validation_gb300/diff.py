"""Differentiable rendering of material parameters on top of the C ABI:
parameter packing (OMV_MATERIAL_PARAMS slots per material), and a
torch.autograd.Function whose forward renders the normalised image
(omv_render_device) and whose backward replays the paths (omv_adjoint).

Slots per material: base colour r, g, b, roughness, metallic (glTF PBR);
n r, g, b, k r, g, b at 650/510/440 nm (OpenMATERIAL conductors)."""
from __future__ import annotations

import ctypes as C
import dataclasses
import importlib
from typing import List

import numpy as np

from . import capi, scenes

SLOTS = 11
PBR_SLOTS = (0, 1, 2, 3, 4)
OM_SLOTS = (5, 6, 7, 8, 9, 10)


def _omv():
    return importlib.import_module("openmaterial-validation_gb300")


def _om_values(m: scenes.Material):
    """n, k at the RGB wavelengths of a conductor's tables (the lookup points)."""
    n = np.interp(scenes.RGB_WAVELENGTHS, m.ior_n[:, 0], m.ior_n[:, 1])
    k = np.interp(scenes.RGB_WAVELENGTHS, m.ior_k[:, 0], m.ior_k[:, 1])
    return n, k


def params_from_materials(materials: List[scenes.Material]) -> np.ndarray:
    P = np.zeros((len(materials), SLOTS), dtype=np.float64)
    for i, m in enumerate(materials):
        if m.type == 0:
            P[i, 0:3] = m.base_color[:3]
            P[i, 3] = m.roughness
            P[i, 4] = m.metallic
        else:
            n, k = _om_values(m)
            P[i, 5:8] = n
            P[i, 8:11] = k
    return P


def active_mask(materials: List[scenes.Material]) -> np.ndarray:
    """Which slots a material type uses."""
    M = np.zeros((len(materials), SLOTS), dtype=bool)
    for i, m in enumerate(materials):
        M[i, list(PBR_SLOTS if m.type == 0 else OM_SLOTS)] = True
    return M


def materials_from_params(materials: List[scenes.Material], P) -> List[scenes.Material]:
    P = np.asarray(P, dtype=np.float64)
    out = []
    for i, m in enumerate(materials):
        if m.type == 0:
            bc = (float(P[i, 0]), float(P[i, 1]), float(P[i, 2]), m.base_color[3])
            out.append(dataclasses.replace(m, base_color=bc, roughness=float(P[i, 3]), metallic=float(P[i, 4])))
        else:
            out.append(scenes._om_conductor(tuple(P[i, 5:8]), tuple(P[i, 8:11]), m.name))
    return out


class MaterialRenderer:
    """Renders one camera of a scene for given material parameters and
    returns its normalised image; with torch, `image(params)` is differentiable
    with respect to `params` (num_materials x 11) through path replay."""

    def __init__(self, scene: scenes.Scene, spp: int, seed: int = 0, adjoint_seed: int = None, device: int = 0):
        omv = _omv()
        self.omv = omv
        self.spec = scene
        self.rs = omv.RenderScene(scene, device)
        self.cam = omv.PinholeCamera.from_spec(scene.camera).to_c()
        self.params = omv.RendererParameters.for_scene(scene, samplesPerPixel=spp, seed=seed).to_c()
        self.adj_params = omv.RendererParameters.for_scene(
            scene, samplesPerPixel=spp, seed=seed if adjoint_seed is None else adjoint_seed).to_c()
        self.materials = list(scene.materials)
        self._keep: list = []

    def set_seeds(self, seed: int, adjoint_seed: int) -> None:
        """Random streams of the next forward render and of the replay."""
        self.params.seed = seed
        self.adj_params.seed = adjoint_seed

    def set_params(self, P) -> None:
        mats = materials_from_params(self.materials, P)
        keep: list = []
        descs = capi.material_descs(mats, keep)
        self.omv.check(self.omv.lib().omv_scene_set_materials(self.rs.handle, len(mats), descs))
        self._keep = keep

    def render_sums(self, torch, stream=None):
        """FP64 film sums (H, W, 3) and counts (H, W) on the device."""
        H, W = self.cam.height, self.cam.width
        s = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
        c = torch.zeros((H, W), dtype=torch.int32, device="cuda")
        st = stream if stream is not None else C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.omv.check(self.omv.lib().omv_render_device(self.rs.handle, C.byref(self.cam), C.byref(self.params),
                                                        C.c_void_p(s.data_ptr()), None, C.c_void_p(c.data_ptr()),
                                                        st, None))
        # the render runs on torch's current stream (NULL: the legacy default
        # stream), so torch reads the film in order; the host waits here so that
        # a caller's timing brackets the render
        torch.cuda.synchronize()
        return s, c

    def adjoint(self, torch, adj_image):
        """d loss / d params for dLoss/dImage `adj_image` (H, W, 3)."""
        a = adj_image.detach().to(device="cuda", dtype=torch.float32).contiguous()
        g = torch.zeros((len(self.materials), SLOTS), dtype=torch.float32, device="cuda")
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.omv.check(self.omv.lib().omv_adjoint(self.rs.handle, C.byref(self.cam), C.byref(self.adj_params),
                                                  C.c_void_p(a.data_ptr()), C.c_void_p(g.data_ptr()), st))
        torch.cuda.synchronize()
        return g

    def image(self, P):
        """Differentiable normalised image (H, W, 3, float64) of parameters P."""
        import torch

        return _RenderFn.apply(P, self)


def _make_fn():
    import torch

    class RenderFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, P, renderer):
            renderer.set_params(P.detach().cpu().numpy())
            s, c = renderer.render_sums(torch)
            ctx.renderer = renderer
            ctx.p_device, ctx.p_dtype = P.device, P.dtype
            return s / c.clamp(min=1).unsqueeze(-1).to(torch.float64)

        @staticmethod
        def backward(ctx, grad_image):
            g = ctx.renderer.adjoint(torch, grad_image)
            return g.to(device=ctx.p_device, dtype=ctx.p_dtype), None

    return RenderFn


class _Lazy:
    fn = None

    def __getattr__(self, name):
        if _Lazy.fn is None:
            _Lazy.fn = _make_fn()
        return getattr(_Lazy.fn, name)


_RenderFn = _Lazy()
