"""Helpers of the GPU tests: device images over torch tensors and one-call
development through the C ABI (libcraw.so)."""
from __future__ import annotations

import numpy as np
import torch

import libcraw_gb300 as L


def pad8(w: int) -> int:
    return (w + 7) // 8 * 8


def upload_mosaic(m: np.ndarray) -> tuple[torch.Tensor, L.Image]:
    """A device copy of an (h, w) uint16 mosaic, rows padded to 16 bytes."""
    h, w = m.shape
    t = torch.zeros((h, pad8(w)), dtype=torch.int16, device="cuda")
    t[:, :w] = torch.from_numpy(m.view(np.int16)).cuda()
    return t, L.Image(t.data_ptr(), t.stride(0) * 2, L.FORMAT_R16_UNORM, w, h)


def alloc_rgba(w: int, h: int, fmt: int = L.FORMAT_RGBA32F) -> tuple[torch.Tensor, L.Image]:
    """A device image of an output format: (h, w, 4) for RGBA32F / RGBA16F,
    (h, w, 3) for RGB32F (rows padded to 16 bytes, the tensor a view of
    them)."""
    if fmt == L.FORMAT_RGB32F:
        pitch = (w * 12 + 15) // 16 * 16
        buf = torch.full((h, pitch // 4), float("nan"), dtype=torch.float32, device="cuda")
        t = buf[:, : 3 * w].view(h, w, 3)
        return t, L.Image(buf.data_ptr(), pitch, fmt, w, h)
    dt = torch.float32 if fmt == L.FORMAT_RGBA32F else torch.float16
    t = torch.full((h, w, 4), float("nan"), dtype=dt, device="cuda")
    return t, L.Image(t.data_ptr(), t.stride(0) * t.element_size(), fmt, w, h)


_cudart_lib = None


def cudart():
    """The CUDA runtime, for copies out of buffers the pipeline owns."""
    global _cudart_lib
    if _cudart_lib is None:
        import ctypes as C
        import glob
        import os
        cands = []
        for d in (os.path.dirname(torch.__file__) + "/lib", "/usr/local/cuda/lib64"):
            cands += sorted(glob.glob(d + "/libcudart.so*"))
        import site
        for sp in site.getsitepackages():
            cands += sorted(glob.glob(sp + "/nvidia/cuda_runtime/lib/libcudart.so*"))
        for c in cands:
            try:
                _cudart_lib = C.CDLL(c)
                break
            except OSError:
                continue
        if _cudart_lib is None:
            raise OSError("libcudart not found")
        _cudart_lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        _cudart_lib.cudaMemcpy.restype = C.c_int
    return _cudart_lib


def download_image(img: L.Image, kind: str) -> np.ndarray:
    """Copies a device image the pipeline owns to the host: kind is
    'rgba32f', 'rgba16f', 'r16', 'r32f' or 'r8'."""
    bpp = {"rgba32f": 16, "rgba16f": 8, "r16": 2, "r16f": 2, "r32f": 4, "r8": 1}[kind]
    torch.cuda.synchronize()
    host = np.empty(img.pitch * img.height, np.uint8)
    ret = cudart().cudaMemcpy(host.ctypes.data, img.data, host.nbytes, 2)  # device to host
    assert ret == 0, ret
    a = host.reshape(img.height, img.pitch)[:, : img.width * bpp]
    dt = {"rgba32f": np.float32, "rgba16f": np.float16, "r16": np.uint16, "r16f": np.float16,
          "r32f": np.float32, "r8": np.uint8}[kind]
    a = np.ascontiguousarray(a).view(dt)
    if kind.startswith("rgba"):
        a = a.reshape(img.height, img.width, 4)
    return a


def develop(pipe: L.Pipeline, m: np.ndarray, fp: L.FrameParams, fmt: int = L.FORMAT_RGBA32F,
            stream: torch.cuda.Stream | None = None) -> np.ndarray:
    h, w = m.shape
    _, src = upload_mosaic(m)
    out, dst = alloc_rgba(w, h, fmt)
    s = stream or torch.cuda.current_stream()
    pipe.record(s.cuda_stream, src, dst, fp)
    torch.cuda.synchronize()
    return out.float().cpu().numpy()
