"""Image development after a render, on the device, over the C ABI: the
reference main's tail (main.cpp:505-521) with the reference's names.

  develop             getImpression after stop + gammaCorrection + 8-bit rgba, one pass
  gammaCorrection     ToneMapping.cpp:24-53, in place
  SimpleDenoiserMedian  Denoiser.h:24-64 (returns a new image)
  rgba8               saveImage's conversion (main.cpp:92)
  saveImage           main.cpp:86-120 with ImageSaver::flipVerticallyOnWrite(true)

Images are torch CUDA tensors of shape (H, W, 4) float32 (or uint8 for rgba8),
contiguous; the calls are enqueued on torch's current stream.
"""
from __future__ import annotations

import ctypes as C
import importlib

import numpy as np


def _omv():
    return importlib.import_module("openmaterial-validation_gb300")


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _check_image(img, dtype_name: str = "float32"):
    if not img.is_cuda or not img.is_contiguous() or img.dim() != 3 or img.shape[2] != 4:
        raise ValueError("expected a contiguous CUDA tensor of shape (H, W, 4)")
    if str(img.dtype) != "torch." + dtype_name:
        raise ValueError(f"expected dtype {dtype_name}")


def develop(sum_rgb, count, gamma: float = 0.5, A: float = 1.0, linear: bool = True, tonemapped: bool = True,
            rgba8: bool = True, flip: bool = True):
    """Film sums (H, W, 3) float64 and counts (H, W) int32/uint32 on the device
    -> dict of the requested images: 'linear' (normalised film), 'tonemapped'
    (gammaCorrection(img, W, H, A, gamma)) and 'rgba8' (rows flipped when flip)."""
    import torch

    omv = _omv()
    H, W = count.shape
    if sum_rgb.shape != (H, W, 3) or sum_rgb.dtype != torch.float64 or not sum_rgb.is_contiguous():
        raise ValueError("sum_rgb must be a contiguous (H, W, 3) float64 tensor")
    dev = sum_rgb.device
    out = {}
    if linear:
        out["linear"] = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    if tonemapped:
        out["tonemapped"] = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    if rgba8:
        out["rgba8"] = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    omv.check(omv.lib().omv_develop(_ptr(sum_rgb), _ptr(count.contiguous()), W, H, A, gamma, _ptr(out.get("linear")),
                                    _ptr(out.get("tonemapped")), _ptr(out.get("rgba8")), 1 if flip else 0,
                                    _stream(torch)))
    return out


def gammaCorrection(img, A: float = 1.0, gamma: float = 0.5):
    """In place, like the reference (ToneMapping.h:25 defaults A=1, gamma=0.5)."""
    import torch

    _check_image(img)
    omv = _omv()
    omv.check(omv.lib().omv_tonemap(_ptr(img), img.shape[0] * img.shape[1], A, gamma, _stream(torch)))
    return img


def SimpleDenoiserMedian(img, half_size: int = 1):
    """The median-filtered image as a new tensor (the reference overwrites its input)."""
    import torch

    _check_image(img)
    out = torch.empty_like(img)
    omv = _omv()
    omv.check(omv.lib().omv_denoise_median(_ptr(img), _ptr(out), img.shape[1], img.shape[0], half_size,
                                           _stream(torch)))
    return out


def rgba8(img, flip: bool = False):
    import torch

    _check_image(img)
    out = torch.empty(img.shape, dtype=torch.uint8, device=img.device)
    omv = _omv()
    omv.check(omv.lib().omv_rgba8(_ptr(img), _ptr(out), img.shape[1], img.shape[0], 1 if flip else 0,
                                  _stream(torch)))
    return out


def saveImage(path: str, img) -> None:
    """Writes an (H, W, 4) float image (numpy, or a tensor copied to the host)
    as .png / .bmp / .tga / .pfm like the reference's saveImage."""
    if hasattr(img, "detach"):
        import torch

        torch.cuda.synchronize()
        img = img.detach().cpu().numpy()
    a = np.ascontiguousarray(img, dtype=np.float32)
    if a.ndim != 3 or a.shape[2] != 4:
        raise ValueError("expected an (H, W, 4) image")
    omv = _omv()
    omv.check(omv.lib().omv_save_image(path.encode(), a.ctypes.data_as(C.POINTER(C.c_float)), a.shape[1], a.shape[0]))
