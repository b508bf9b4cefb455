"""torch.autograd.Function over the C ABI: a differentiable render of the
float image with respect to the material table's albedo and emission and the
camera position.

Forward: tracer_trace (RGBA32F and LINEAR AOVs).  Backward: tracer_trace_adjoint
(path replay) with the forward's LINEAR image, writing the gradients straight
into torch device tensors.  The tracer's stream work is ordered with torch's
by synchronising around each call.
"""
from __future__ import annotations

import numpy as np
import torch

from . import abi
from . import scene as S


class _DeviceView:
    """__cuda_array_interface__ over a device buffer owned by the tracer."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"data": (ptr, False), "shape": tuple(shape), "typestr": typestr,
                                         "version": 3, "strides": None}


class DifferentiableRenderer:
    """A tracer with an uploaded triangle scene whose material table and
    camera position are the differentiable inputs."""

    def __init__(self, tracer: abi.Tracer, scene: S.Scene, frame: np.ndarray, params: abi.TraceParams):
        self.tr = tracer
        self.scene = scene
        self.frame = np.array(frame, S.FRAME).reshape(())
        self.params = params
        self.params.aov_mask = (1 << abi.AOV_RGBA32F) | (1 << abi.AOV_LINEAR)
        self.materials = np.array(scene.materials, S.MATERIAL)
        tracer.upload_scene(scene)

    @property
    def num_materials(self) -> int:
        return len(self.materials)

    def _apply(self, albedo: torch.Tensor, emission: torch.Tensor, campos: torch.Tensor):
        m = self.materials.copy()
        m["albedo"] = albedo.detach().to("cpu", torch.float32).numpy()
        m["emissive"] = emission.detach().to("cpu", torch.float32).numpy()
        self.tr.set_materials(m)
        f = self.frame.copy()
        f["camera"]["pos"] = campos.detach().to("cpu", torch.float32).numpy()
        return f

    def render(self, albedo: torch.Tensor, emission: torch.Tensor, campos: torch.Tensor) -> torch.Tensor:
        """(h, w, 3) float image (RGBA32F without alpha) on the GPU."""
        return _Render.apply(albedo, emission, campos, self)


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo, emission, campos, r: DifferentiableRenderer):
        f = r._apply(albedo, emission, campos)
        p = r.params
        torch.cuda.synchronize()
        r.tr.trace(f, p)
        r.tr.synchronize()
        ptr, _ = r.tr.device_image(abi.AOV_RGBA32F)
        img = torch.as_tensor(_DeviceView(ptr, (p.height, p.width, 4), "<f4"), device="cuda").clone()
        lptr, _ = r.tr.device_image(abi.AOV_LINEAR)
        lin = torch.as_tensor(_DeviceView(lptr, (p.height, p.width, 4), "<f4"), device="cuda").clone()
        ctx.r = r
        ctx.frame = f
        ctx.save_for_backward(lin)
        return img[..., :3]

    @staticmethod
    def backward(ctx, grad_img):
        (lin,) = ctx.saved_tensors
        r = ctx.r
        p = r.params
        dl = torch.zeros((p.height, p.width, 4), dtype=torch.float32, device="cuda")
        dl[..., :3] = grad_img
        nm = r.num_materials
        ga = torch.zeros((nm, 3), dtype=torch.float32, device="cuda")
        ge = torch.zeros((nm, 3), dtype=torch.float32, device="cuda")
        gc = torch.zeros(3, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        r.tr.trace_adjoint(ctx.frame, p, dl.data_ptr(), lin.data_ptr(),
                           outputs=(ga.data_ptr(), ge.data_ptr(), gc.data_ptr()))
        r.tr.synchronize()
        return ga, ge, gc, None
