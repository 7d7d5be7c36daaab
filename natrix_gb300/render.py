"""Headless visualisation: the reference demo's display shaders as CUDA
kernels writing device buffers (demo/shaders/demo.ComputeShader.comp,
demo.FieldFragmentShader.frag, demo.QuiverFragmentShader.frag), plus a PNG
writer for saving a frame.  No graphics pipeline is involved: each output is
an RGBA8 (H, W, 4) uint8 CUDA tensor, R first.
"""
from __future__ import annotations

import ctypes
import struct
import zlib
from typing import Optional, Tuple

import numpy as np
import torch

from ._lib import call


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _as_field(t: torch.Tensor, comps: int) -> Tuple[int, int, int]:
    """(height, width, row pitch in elements) of a float32 CUDA field view."""
    if not t.is_cuda or t.dtype != torch.float32:
        raise ValueError("expected a float32 CUDA tensor")
    if comps == 1:
        if t.dim() != 2 or t.stride(1) != 1:
            raise ValueError("expected an (H, W) field with unit column stride")
        return t.shape[0], t.shape[1], t.stride(0)
    if t.dim() != 3 or t.shape[2] != 2 or t.stride(2) != 1 or t.stride(1) != 2 \
            or t.stride(0) % 2:
        raise ValueError("expected an (H, W, 2) velocity with interleaved components")
    return t.shape[0], t.shape[1], t.stride(0) // 2


def render_density(density, texture: bool = True, colour: bool = True):
    """Density -> (texture, colour) RGBA8 tensors (either may be None).

    ``density`` is a SmoothParticlesArea or an (H, W) float32 CUDA field.
    texture: the demo's compute shader (imageStore of vec4(rho) into rgba8);
    colour: the field shader's vec4(plasma(fbm(c)), c), one pixel per cell."""
    field = density.density if hasattr(density, "density") else density
    H, W, pitch = _as_field(field, 1)
    tex = torch.empty(H, W, 4, dtype=torch.uint8, device=field.device) if texture else None
    col = torch.empty(H, W, 4, dtype=torch.uint8, device=field.device) if colour else None
    call("natrix_render_density", ctypes.c_void_p(field.data_ptr()), W, H, pitch,
         ctypes.c_void_p(tex.data_ptr() if tex is not None else None),
         ctypes.c_void_p(col.data_ptr() if col is not None else None), W, _stream())
    return tex, col


def quiver_tiles(window: Tuple[int, int], tile: float) -> Tuple[int, int]:
    nx, ny = ctypes.c_int32(), ctypes.c_int32()
    call("natrix_quiver_tiles", int(window[0]), int(window[1]), float(tile), ctypes.byref(nx),
         ctypes.byref(ny))
    return nx.value, ny.value


def quiver(velocity, window: Optional[Tuple[int, int]] = None, tile: float = 16.0,
           overlay: bool = True):
    """Quiver plot of a velocity field: (arrows (ny, nx, 2) float32 in window
    pixels, overlay (win_h, win_w, 4) RGBA8 or None).

    ``velocity`` is a FluidSimulator or an (H, W, 2) float32 CUDA view;
    ``window`` (width, height) defaults to twice the grid, as the demo draws
    it; ``tile`` is the arrow tile size in pixels (the demo offers 8, 16, 32,
    64)."""
    v = velocity.get_velocity_buffer() if hasattr(velocity, "get_velocity_buffer") else velocity
    H, W, pitch = _as_field(v, 2)
    if window is None:
        window = (2 * W, 2 * H)
    nx, ny = quiver_tiles(window, tile)
    arrows = torch.empty(ny, nx, 2, dtype=torch.float32, device=v.device)
    ov = None
    if overlay:
        ov = torch.empty(int(window[1]), int(window[0]), 4, dtype=torch.uint8, device=v.device)
    call("natrix_quiver", ctypes.c_void_p(v.data_ptr()), W, H, pitch, int(window[0]),
         int(window[1]), float(tile), ctypes.c_void_p(arrows.data_ptr()),
         ctypes.c_void_p(ov.data_ptr() if ov is not None else None), int(window[0]), _stream())
    return arrows, ov


def blend_over(top: torch.Tensor, bottom: torch.Tensor) -> torch.Tensor:
    """Source-over alpha blend of two RGBA8 frames of equal size (the demo
    draws the quiver overlay over the field with alpha blending)."""
    a = top[..., 3:4].float() / 255.0
    rgb = top[..., :3].float() * a + bottom[..., :3].float() * (1.0 - a)
    out = bottom.clone()
    out[..., :3] = rgb.round().clamp(0, 255).to(torch.uint8)
    return out


def write_png(path, rgba) -> None:
    """Write an (H, W, 4) uint8 frame (tensor or array) as an RGBA PNG."""
    img = rgba.cpu().numpy() if hasattr(rgba, "cpu") else np.asarray(rgba)
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape[:2]
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(H))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return (struct.pack(">I", len(data)) + tag + data
                + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF))

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


__all__ = ["render_density", "quiver", "quiver_tiles", "blend_over", "write_png"]
