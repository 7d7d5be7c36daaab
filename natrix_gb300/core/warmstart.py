"""Learned pressure warm start: a small U-Net that predicts the converged
pressure of a step from its divergence and obstacle mask, so the Jacobi
sweeps start close to the solution.  No reference counterpart: the reference
starts every solve from zero (natrix/core/fluid_simulator.py:235-248).

Network (NHWC bf16 activations, FP32 master weights, Adam):
  level 1 (H x W):      conv 2->16, conv 16->16                 -> e1
  level 2 (H/2):        avgpool, conv 16->32, conv 32->32       -> e2
  level 3 (H/4):        avgpool, conv 32->64, conv 64->64       -> e3
  decoder level 2:      up(e3) ++ e2 -> conv 96->32, conv 32->32 -> d2
  decoder level 1:      up(d2) ++ e1 -> conv 48->16, conv 16->16 -> d1
  head:                 1x1 conv 16->1                           -> p
Every 3x3 conv is followed by ReLU and runs as a tcgen05 implicit GEMM
(natrix_nn_conv3x3); input gradients run through the same kernel with
flipped weights, weight gradients on CUDA cores (natrix_nn_wgrad).

Units: the network sees div / s and predicts p / s, s = RMS of the
divergence over the fluid cells of the image (the pressure equation is
linear, so the scale is exact).

Loss (natrix_nn_loss): mean squared mean-removed pressure error over fluid
cells plus lambda times the squared residual of the sweep's operator,
relative to the squared right-hand side.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from .. import _lib

_F = ctypes.c_float
_I = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
_P = ctypes.c_void_p


class NnConv(ctypes.Structure):
    _fields_ = [("src0", _P), ("c0", _I), ("src1", _P), ("c1", _I), ("B", _I), ("H", _I),
                ("W", _I), ("N", _I), ("wpack", _P), ("bias", _P), ("relu", _I), ("gate", _P),
                ("out0", _P), ("n0", _I), ("out1", _P), ("head_w", _P), ("head_b", _F),
                ("head_out", _P), ("status", _P)]


_SIGS = {
    "natrix_nn_conv3x3": [ctypes.POINTER(NnConv), _P],
    "natrix_nn_pack": [_P, _I, _I, _I, _I, _I, _P, _P],
    "natrix_nn_wgrad": [_P, _I, _P, _I, _P, _I, _I, _I, _I, _P, _P, _P],
    "natrix_nn_wgrad_status": [ctypes.POINTER(ctypes.c_int32)],
    "natrix_nn_prep": [_P, _P, _P, _I, _I, _I, _I, _P, _P],
    "natrix_nn_pool": [_P, _I, _I, _I, _I, _P, _P],
    "natrix_nn_up": [_P, _I, _I, _I, _I, _P, _P],
    "natrix_nn_up_back": [_P, _I, _I, _I, _I, _P, _P, _P],
    "natrix_nn_pool_back": [_P, _P, _I, _I, _I, _I, _P, _P, _P],
    "natrix_nn_head_back": [_P, _P, _I, _I64, _P, _P, _P, _P, _P],
    "natrix_nn_loss": [_P, _P, _P, _P, _P, _I, _I, _I, _I, _F, _P, _P, _P, _P],
    "natrix_nn_adam": [_P, _P, _P, _P, _I64, _F, _F, _F, _F, _I, _P],
    "natrix_nn_cg_apply": [_P, _P, _I, _I, _I, _I, _P, _P],
    "natrix_nn_cg_dot": [_P, _P, _P, _I, _I, _I, _I, _P, _P],
    "natrix_nn_cg_axpy": [_P, _P, _P, _P, _D, _I, _I64, _P],
    "natrix_nn_cg_dir": [_P, _P, _P, _P, _I, _I64, _P],
    "natrix_nn_cg_apply_dot": [_P, _P, _I, _I, _I, _I, _P, _P, _P],
    "natrix_nn_cg_update": [_P, _P, _P, _P, _P, _P, _P, _I, _I64, _P],
}
_bound = False


def _lib_nn():
    global _bound
    lib = _lib.load()
    if not _bound:
        for name, args in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _bound = True
    return lib


def _call(name, *args):
    _lib.check(getattr(_lib_nn(), name)(*args))


def _p(t: Optional[torch.Tensor]):
    return _P(t.data_ptr()) if t is not None else None


def _s():
    return _P(torch.cuda.current_stream().cuda_stream)


# (name, c0, c1, cout): c0 / c1 = channels of the two concatenated sources
LAYERS = [("c11", 8, 0, 16), ("c12", 16, 0, 16), ("c21", 16, 0, 32), ("c22", 32, 0, 32),
          ("c31", 32, 0, 64), ("c32", 64, 0, 64), ("c41", 64, 32, 32), ("c42", 32, 0, 32),
          ("c51", 32, 16, 16), ("c52", 16, 0, 16)]
# real input channels of the first layer (divergence, obstacle); the rest of
# its 8 input channels are zero
REAL_IN = {"c11": 2}


def _r16(n: int) -> int:
    return (n + 15) // 16 * 16


@dataclass
class Layer:
    name: str
    c0: int
    c1: int
    cout: int
    cin: int          # master-weight input channels
    w: torch.Tensor   # FP32 [cout][cin][3][3]
    b: torch.Tensor   # FP32 [cout]
    gw: torch.Tensor
    gb: torch.Tensor
    mw: torch.Tensor
    vw: torch.Tensor
    mb: torch.Tensor
    vb: torch.Tensor
    fwd: torch.Tensor  # packed bf16 operands (uint16 storage)
    bwd: torch.Tensor


class UNet:
    """The warm-start network on the GPU (parameters, activations, Adam)."""

    def __init__(self, seed: int = 0, device: str = "cuda"):
        self.device = device
        g = torch.Generator().manual_seed(seed)
        self.layers: list[Layer] = []
        for name, c0, c1, cout in LAYERS:
            cin = REAL_IN.get(name, c0 + c1)
            std = math.sqrt(2.0 / (9 * cin))
            w = (torch.randn(cout, cin, 3, 3, generator=g, dtype=torch.float64) * std).float()
            ctot = _r16(c0 + c1)
            z = lambda *s: torch.zeros(*s, dtype=torch.float32, device=device)  # noqa: E731
            lay = Layer(name, c0, c1, cout, cin, w.to(device), z(cout), z(cout, cin, 3, 3), z(cout),
                        z(cout, cin, 3, 3), z(cout, cin, 3, 3), z(cout), z(cout),
                        torch.zeros(cout * 9 * ctot, dtype=torch.int16, device=device),
                        torch.zeros(_r16(c0 + c1) * 9 * cout, dtype=torch.int16, device=device))
            self.layers.append(lay)
        self.hw = (torch.randn(16, generator=g, dtype=torch.float64) * math.sqrt(1 / 16)).float().to(device)
        self.hb = torch.zeros(1, dtype=torch.float32, device=device)
        self.ghw = torch.zeros_like(self.hw)
        self.ghb = torch.zeros_like(self.hb)
        self.mhw, self.vhw = torch.zeros_like(self.hw), torch.zeros_like(self.hw)
        self.mhb, self.vhb = torch.zeros_like(self.hb), torch.zeros_like(self.hb)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        # fixed output multiplier: p = out_scale * (hw . d1 + hb), set from the
        # RMS of the training targets so the head's weights stay O(1)
        self.out_scale = 1.0
        self._ghw_eff = torch.zeros_like(self.hw)
        self._ghb_eff = torch.zeros_like(self.hb)
        self.step_count = 0
        self.repack()
        self.acts: dict[str, torch.Tensor] = {}
        self.shape = None

    # ------------------------------------------------------------ parameters
    def repack(self):
        for L in self.layers:
            ctot = _r16(L.c0 + L.c1)
            _call("natrix_nn_pack", _p(L.w), L.cout, L.cin, L.cout, ctot, 0, _p(L.fwd), _s())
            _call("natrix_nn_pack", _p(L.w), L.cout, L.cin, _r16(L.c0 + L.c1), L.cout, 1,
                  _p(L.bwd), _s())

    def parameters(self):
        out = []
        for L in self.layers:
            out += [(L.w, L.gw, L.mw, L.vw), (L.b, L.gb, L.mb, L.vb)]
        out += [(self.hw, self.ghw, self.mhw, self.vhw), (self.hb, self.ghb, self.mhb, self.vhb)]
        return out

    def state_dict(self) -> dict:
        d = {f"{L.name}.w": L.w.cpu() for L in self.layers}
        d.update({f"{L.name}.b": L.b.cpu() for L in self.layers})
        d["head.w"], d["head.b"] = self.hw.cpu(), self.hb.cpu()
        d["out_scale"] = torch.tensor(self.out_scale)
        return d

    def load_state_dict(self, d: dict) -> None:
        for L in self.layers:
            L.w.copy_(d[f"{L.name}.w"])
            L.b.copy_(d[f"{L.name}.b"])
        self.hw.copy_(d["head.w"])
        self.hb.copy_(d["head.b"])
        self.out_scale = float(d.get("out_scale", torch.tensor(1.0)))
        self.repack()

    def zero_grad(self):
        for _, g, _, _ in self.parameters():
            g.zero_()

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for w, g, m, v in self.parameters():
            _call("natrix_nn_adam", _p(w), _p(g), _p(m), _p(v), w.numel(), lr, b1, b2, eps,
                  self.step_count, _s())
        self.repack()

    # ---------------------------------------------------------------- buffers
    def _alloc(self, B, H, W):
        if self.shape == (B, H, W):
            return
        dev = self.device
        bf = lambda h, w, c: torch.empty(B, h, w, c, dtype=torch.int16, device=dev)  # noqa: E731
        H2, W2, H4, W4 = H // 2, W // 2, H // 4, W // 4
        a = {}
        a["x"] = bf(H, W, 8)
        a["a11"], a["e1"] = bf(H, W, 16), bf(H, W, 16)
        a["q1"] = bf(H2, W2, 16)
        a["a21"], a["e2"] = bf(H2, W2, 32), bf(H2, W2, 32)
        a["q2"] = bf(H4, W4, 32)
        a["a31"], a["e3"] = bf(H4, W4, 64), bf(H4, W4, 64)
        a["u3"] = bf(H2, W2, 64)
        a["a41"], a["d2"] = bf(H2, W2, 32), bf(H2, W2, 32)
        a["u2"] = bf(H, W, 32)
        a["a51"], a["d1"] = bf(H, W, 16), bf(H, W, 16)
        # gradients (reuse-free for clarity; sizes are modest)
        a["g16"], a["h16"] = bf(H, W, 16), bf(H, W, 16)
        a["gu2"] = bf(H, W, 32)
        a["ge1s"] = bf(H, W, 16)
        a["g32"], a["h32"] = bf(H2, W2, 32), bf(H2, W2, 32)
        a["gu3"] = bf(H2, W2, 64)
        a["ge2s"] = bf(H2, W2, 32)
        a["gq1"] = bf(H2, W2, 16)
        a["g64"], a["h64"] = bf(H4, W4, 64), bf(H4, W4, 64)
        a["gq2"] = bf(H4, W4, 32)
        a["p"] = torch.empty(B, H, W, dtype=torch.float32, device=dev)
        a["dp"] = torch.empty_like(a["p"])
        a["r"] = torch.empty_like(a["p"])
        a["sums"] = torch.empty(B, 6, dtype=torch.float64, device=dev)
        self.acts = a
        self.shape = (B, H, W)

    def _conv(self, L: Layer, src0, src1, B, H, W, out0, relu=True, gate=None, out1=None, n0=0,
              head_out=None, backward=False):
        c = NnConv()
        if not backward:
            c.src0, c.c0 = _p(src0), L.c0
            c.src1, c.c1 = _p(src1), L.c1 if src1 is not None else 0
            c.N, c.wpack, c.bias, c.relu = L.cout, _p(L.fwd), _p(L.b), 1 if relu else 0
        else:
            c.src0, c.c0, c.src1, c.c1 = _p(src0), L.cout, None, 0
            c.N, c.wpack, c.bias, c.relu = _r16(L.c0 + L.c1), _p(L.bwd), None, 0
        c.B, c.H, c.W = B, H, W
        c.gate = _p(gate)
        c.out0, c.n0, c.out1 = _p(out0), n0, _p(out1)
        if head_out is not None:
            self._hw_eff = self.hw * self.out_scale
            c.head_w = _p(self._hw_eff)
            c.head_b = float(self.hb.item()) * self.out_scale
            c.head_out = _p(head_out)
        c.status = _p(self.status)
        _call("natrix_nn_conv3x3", ctypes.byref(c), _s())

    # ----------------------------------------------------------------- forward
    def forward(self, div: torch.Tensor, mask: Optional[torch.Tensor], inv_scale: torch.Tensor,
                H: int, W: int, pitch: int) -> torch.Tensor:
        """div: B pitched float fields (B*H*pitch), mask: uint8 same layout or
        None, inv_scale: B floats.  Returns p / s (B x H x W float32)."""
        B = inv_scale.numel()
        if H % 4 or W % 4:
            raise ValueError("grid sides must be multiples of 4")
        self._alloc(B, H, W)
        a = self.acts
        L = {l.name: l for l in self.layers}
        H2, W2, H4, W4 = H // 2, W // 2, H // 4, W // 4
        _call("natrix_nn_prep", _p(div), _p(mask), _p(inv_scale), B, H, W, pitch, _p(a["x"]), _s())
        self._conv(L["c11"], a["x"], None, B, H, W, a["a11"])
        self._conv(L["c12"], a["a11"], None, B, H, W, a["e1"])
        _call("natrix_nn_pool", _p(a["e1"]), B, H, W, 16, _p(a["q1"]), _s())
        self._conv(L["c21"], a["q1"], None, B, H2, W2, a["a21"])
        self._conv(L["c22"], a["a21"], None, B, H2, W2, a["e2"])
        _call("natrix_nn_pool", _p(a["e2"]), B, H2, W2, 32, _p(a["q2"]), _s())
        self._conv(L["c31"], a["q2"], None, B, H4, W4, a["a31"])
        self._conv(L["c32"], a["a31"], None, B, H4, W4, a["e3"])
        _call("natrix_nn_up", _p(a["e3"]), B, H4, W4, 64, _p(a["u3"]), _s())
        self._conv(L["c41"], a["u3"], a["e2"], B, H2, W2, a["a41"])
        self._conv(L["c42"], a["a41"], None, B, H2, W2, a["d2"])
        _call("natrix_nn_up", _p(a["d2"]), B, H2, W2, 32, _p(a["u2"]), _s())
        self._conv(L["c51"], a["u2"], a["e1"], B, H, W, a["a51"])
        self._conv(L["c52"], a["a51"], None, B, H, W, a["d1"], head_out=a["p"])
        return a["p"]

    # ---------------------------------------------------------------- backward
    def backward(self, dp: torch.Tensor):
        """Accumulate parameter gradients for the last forward, given dL/dp."""
        B, H, W = self.shape
        a = self.acts
        L = {l.name: l for l in self.layers}
        H2, W2, H4, W4 = H // 2, W // 2, H // 4, W // 4
        n = B * H * W
        wg = lambda lay, dz, x0, x1, h, w: _call(  # noqa: E731
            "natrix_nn_wgrad", _p(dz), lay.cout, _p(x0), lay.c0, _p(x1),
            lay.c1 if x1 is not None else 0, B, h, w, _p(lay.gw), _p(lay.gb), _s())
        self._ghw_eff.zero_()
        self._ghb_eff.zero_()
        _call("natrix_nn_head_back", _p(dp), _p(a["d1"]), 16, n, _p(self._hw_eff),
              _p(self._ghw_eff), _p(self._ghb_eff), _p(a["g16"]), _s())
        self.ghw += self._ghw_eff * self.out_scale
        self.ghb += self._ghb_eff * self.out_scale
        # c52: dz52 = g16
        wg(L["c52"], a["g16"], a["a51"], None, H, W)
        self._conv(L["c52"], a["g16"], None, B, H, W, a["h16"], gate=a["a51"], backward=True)
        # c51: dz51 = h16 -> [du2 (32), de1 skip (16)]
        wg(L["c51"], a["h16"], a["u2"], a["e1"], H, W)
        self._conv(L["c51"], a["h16"], None, B, H, W, a["gu2"], out1=a["ge1s"], n0=32,
                   backward=True)
        _call("natrix_nn_up_back", _p(a["gu2"]), B, H2, W2, 32, _p(a["d2"]), _p(a["g32"]), _s())
        # c42: dz42 = g32
        wg(L["c42"], a["g32"], a["a41"], None, H2, W2)
        self._conv(L["c42"], a["g32"], None, B, H2, W2, a["h32"], gate=a["a41"], backward=True)
        # c41: dz41 = h32 -> [du3 (64), de2 skip (32)]
        wg(L["c41"], a["h32"], a["u3"], a["e2"], H2, W2)
        self._conv(L["c41"], a["h32"], None, B, H2, W2, a["gu3"], out1=a["ge2s"], n0=64,
                   backward=True)
        _call("natrix_nn_up_back", _p(a["gu3"]), B, H4, W4, 64, _p(a["e3"]), _p(a["g64"]), _s())
        # c32: dz32 = g64
        wg(L["c32"], a["g64"], a["a31"], None, H4, W4)
        self._conv(L["c32"], a["g64"], None, B, H4, W4, a["h64"], gate=a["a31"], backward=True)
        # c31: dz31 = h64 -> dq2
        wg(L["c31"], a["h64"], a["q2"], None, H4, W4)
        self._conv(L["c31"], a["h64"], None, B, H4, W4, a["gq2"], backward=True)
        # e2: (skip + pool gradient) * (e2 > 0) -> dz22 (g32 reused)
        _call("natrix_nn_pool_back", _p(a["ge2s"]), _p(a["gq2"]), B, H2, W2, 32, _p(a["e2"]),
              _p(a["g32"]), _s())
        wg(L["c22"], a["g32"], a["a21"], None, H2, W2)
        self._conv(L["c22"], a["g32"], None, B, H2, W2, a["h32"], gate=a["a21"], backward=True)
        # c21: dz21 = h32 -> dq1
        wg(L["c21"], a["h32"], a["q1"], None, H2, W2)
        self._conv(L["c21"], a["h32"], None, B, H2, W2, a["gq1"], backward=True)
        _call("natrix_nn_pool_back", _p(a["ge1s"]), _p(a["gq1"]), B, H, W, 16, _p(a["e1"]),
              _p(a["g16"]), _s())
        wg(L["c12"], a["g16"], a["a11"], None, H, W)
        self._conv(L["c12"], a["g16"], None, B, H, W, a["h16"], gate=a["a11"], backward=True)
        # the input tensor carries 8 channels, the first layer's weights only
        # the real ones: accumulate into a full-width buffer, keep those
        c11 = L["c11"]
        if not hasattr(self, "_gw11"):
            self._gw11 = torch.zeros(c11.cout, 8, 3, 3, dtype=torch.float32, device=self.device)
        self._gw11.zero_()
        _call("natrix_nn_wgrad", _p(a["h16"]), c11.cout, _p(a["x"]), 8, None, 0, B, H, W,
              _p(self._gw11), _p(c11.gb), _s())
        c11.gw += self._gw11[:, :c11.cin]

    def check_status(self):
        wg = ctypes.c_int32(0)
        _call("natrix_nn_wgrad_status", ctypes.byref(wg))
        if int(self.status.item()) != 0 or wg.value != 0:
            self.status.zero_()
            raise _lib.NatrixError(_lib.NATRIX_EDEVICE, "a tensor-core wait ran out")

    # -------------------------------------------------------------- training
    def loss(self, target: torch.Tensor, div: torch.Tensor, mask, inv_scale, pitch: int,
             lam: float = 1.0, grad: bool = True) -> float:
        B, H, W = self.shape
        a = self.acts
        _call("natrix_nn_loss", _p(a["p"]), _p(target), _p(div), _p(inv_scale), _p(mask), B, H,
              W, pitch, lam, _p(a["sums"]), _p(a["r"]), _p(a["dp"]) if grad else None, _s())
        s = a["sums"].double()
        n = s[:, 0].clamp(min=1)
        lp = s[:, 2] / n - (s[:, 1] / n) ** 2
        lr_ = s[:, 3] / s[:, 4].clamp(min=1e-300)
        return float((lp + lam * lr_).mean().item())

    def train_step(self, div, mask, inv_scale, target, H, W, pitch, lr=1e-3, lam=1.0) -> float:
        self.forward(div, mask, inv_scale, H, W, pitch)
        loss = self.loss(target, div, mask, inv_scale, pitch, lam, grad=True)
        self.zero_grad()
        self.backward(self.acts["dp"])
        self.adam(lr=lr)
        return loss


# ------------------------------------------------------------- cost model
def forward_cost(B: int, H: int, W: int) -> tuple:
    """(tensor-core FLOPs, algorithmic HBM bytes) of one ``UNet.forward`` on
    B images of H x W: every kernel reads its inputs once and writes its
    outputs once (bf16 activations, 2 bytes per channel).  Per full-resolution
    pixel: prep 21, c11 48, c12 64, pool 40, c21 24, c22 32, pool 20, c31 12,
    c32 16, up 40, c41 64, c42 32, up 80, c51 128, c52 + head 68: 689 bytes.
    FLOPs count the padded K the tensor cores execute (input channels rounded
    up to 16)."""
    p1 = B * H * W
    flops = 0.0
    for name, c0, c1, cout in LAYERS:
        level = {"c1": 1, "c2": 2, "c3": 4, "c4": 2, "c5": 1}[name[:2]]
        flops += 2.0 * (p1 // (level * level)) * 9 * _r16(c0 + c1) * cout
    return flops, 689.0 * p1


# ------------------------------------------------------------------ targets
def inv_scale_of(div: torch.Tensor, mask: Optional[torch.Tensor]) -> torch.Tensor:
    """1 / RMS of the divergence over fluid cells, per image (B x H x pitch)."""
    d = div.double()
    if mask is not None:
        f = (mask == 0).double()
        ms = (d * d * f).sum(dim=(1, 2)) / f.sum(dim=(1, 2)).clamp(min=1)
    else:
        ms = (d * d).mean(dim=(1, 2))
    return (1.0 / ms.clamp(min=1e-30).sqrt()).float()


class Regions:
    """Connected fluid regions (4-connected, the stencil's neighbours) of B
    obstacle masks, numbered across the batch: ``labels`` int64 B x H x W
    (-1 on obstacle cells), ``n`` regions, ``count`` cells per region.  The
    pressure operator restricted to fluid cells is pure Neumann on every
    region (obstacle neighbours and walls mirror the centre), so its null
    space is one constant per region and a right-hand side is solvable only
    with each region's mean removed."""

    def __init__(self, mask: Optional[torch.Tensor], B: int, H: int, W: int, device="cuda"):
        from scipy import ndimage

        if mask is None:
            lab = np.broadcast_to(np.arange(B, dtype=np.int64).reshape(B, 1, 1), (B, H, W))
            n = B
        else:
            m = mask[:, :, :W].cpu().numpy()
            lab = np.empty((B, H, W), np.int64)
            n = 0
            for b in range(B):
                l, k = ndimage.label(m[b] == 0)
                lab[b] = np.where(l > 0, l.astype(np.int64) - 1 + n, -1)
                n += k
        self.n = max(n, 1)
        self.labels = torch.from_numpy(np.ascontiguousarray(lab)).to(device)
        self.fluid = self.labels >= 0
        self._idx = self.labels.clamp(min=0).view(-1)
        ones = self.fluid.double().view(-1)
        self.count = torch.zeros(self.n, dtype=torch.float64, device=device).index_add_(
            0, self._idx, ones)

    def project(self, v: torch.Tensor) -> torch.Tensor:
        """v (B x H x W, float64) with each region's mean removed; 0 on obstacles."""
        f = self.fluid.view(-1)
        flat = torch.where(f, v.reshape(-1), torch.zeros((), dtype=v.dtype, device=v.device))
        sums = torch.zeros(self.n, dtype=v.dtype, device=v.device).index_add_(0, self._idx, flat)
        mean = sums / self.count.clamp(min=1)
        return torch.where(f, flat - mean[self._idx], torch.zeros_like(flat)).view_as(v)

    def image_labels(self, b: int) -> tuple:
        """Labels of image b renumbered from 0 (int32, for natrix_residual_regions)."""
        lab = self.labels[b]
        lo = int(lab[lab >= 0].min().item()) if bool((lab >= 0).any()) else 0
        hi = int(lab.max().item())
        out = torch.where(lab >= 0, lab - lo, torch.full_like(lab, -1)).to(torch.int32)
        return out.contiguous(), max(hi - lo + 1, 1)


def cg_solve(div: torch.Tensor, mask: Optional[torch.Tensor], inv_scale: torch.Tensor, H: int,
             W: int, pitch: int, rtol: float = 1e-6, max_iter: int = 20000, check: int = 25,
             regions: Optional[Regions] = None, as_double: bool = False):
    """FP64 conjugate gradients for A p = div * inv_scale on the fluid cells
    of B images (A = the sweep's operator, symmetric negative semidefinite on
    the fluid cells).  The right-hand side is projected onto the range of A
    (each connected fluid region's mean removed), so CG converges; the
    solution is mean-free per region.  Returns (p float32 B x H x W,
    relative residuals B, iterations)."""
    B = inv_scale.numel()
    dev = div.device
    if regions is None:
        regions = Regions(mask, B, H, W, dev)
    dense = div[:, :, :W].double() * inv_scale.double().view(B, 1, 1)
    c = regions.project(-dense).contiguous()
    x = torch.zeros_like(c)
    r = c.clone()
    d = r.clone()
    q = torch.empty_like(c)
    rr = torch.empty(B, dtype=torch.float64, device=dev)
    rr_new = torch.empty_like(rr)
    dq = torch.empty_like(rr)
    cc = torch.empty_like(rr)
    mp = _p(mask) if mask is not None else None
    per = H * W
    _call("natrix_nn_cg_dot", _p(c), _p(c), mp, B, H, W, pitch, _p(cc), _s())
    _call("natrix_nn_cg_dot", _p(r), _p(r), mp, B, H, W, pitch, _p(rr), _s())
    it = 0
    rel = torch.ones(B, dtype=torch.float64)
    while it < max_iter:
        # q = -A d and d.q; x += a d, r -= a q and r.r (a = rr / d.q); d = r + b d
        _call("natrix_nn_cg_apply_dot", _p(d), mp, B, H, W, pitch, _p(q), _p(dq), _s())
        _call("natrix_nn_cg_update", _p(x), _p(r), _p(d), _p(q), _p(rr), _p(dq), _p(rr_new), B,
              per, _s())
        _call("natrix_nn_cg_dir", _p(d), _p(r), _p(rr_new), _p(rr), B, per, _s())
        rr, rr_new = rr_new, rr
        it += 1
        if it % check == 0:
            rel = (rr / cc.clamp(min=1e-300)).sqrt().cpu()
            if float(rel.max()) <= rtol:
                break
    # true relative residual (per-region mean removed), from the final iterate
    _call("natrix_nn_cg_apply", _p(x), mp, B, H, W, pitch, _p(q), _s())
    res = regions.project(c - q)
    true_rel = (res.pow(2).sum(dim=(1, 2)) / cc.clamp(min=1e-300)).sqrt().cpu()
    x = regions.project(x)
    return (x if as_double else x.float()), true_rel, it


# --------------------------------------------------------------- data, eval
@dataclass
class PairSet:
    """(divergence, obstacle mask) -> converged pressure pairs, on the device.
    div / mask: B x H x pitch (the solver's pitched layout); target: B x H x W
    in divergence-normalised units; inv_scale: B."""

    div: torch.Tensor
    mask: torch.Tensor
    inv_scale: torch.Tensor
    target: torch.Tensor
    rel_residual: torch.Tensor
    cg_iterations: int

    @property
    def n(self) -> int:
        return self.inv_scale.numel()


def solver_snapshots(size: int, n: int, seed: int, steps_between: int = 3,
                     reobstacle_every: int = 8):
    """Run the solver on a size x size grid with the large workload's settings
    (eps 0.35, 12 discs, 16 Gaussian splats per step) and record n (div, mask)
    pairs, each after `steps_between` steps; new obstacles every
    `reobstacle_every` pairs."""
    from .. import workloads as wl
    from .fluid_simulator import FluidSimulator

    sim = FluidSimulator(size, size)
    sim.iterations, sim.vorticity, sim.viscosity, sim.speed, sim.dissipation = 80, 0.35, 0.0, 5.0, 0.99
    rng = np.random.default_rng(seed)
    divs, masks = [], []
    obst = None
    for k in range(n):
        if k % reobstacle_every == 0:
            obst = wl.circle_obstacles(rng, 12, size, size)
        for s in range(steps_between):
            for o in obst:
                sim.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
            if s == steps_between - 1:
                mask = sim.obstacles.clone()  # rasterised for the coming step
            sim.add_splats(wl.gauss_splats(rng, 16, size, size, 5.0))
            sim.update(1 / 60)
        divs.append(sim.divergence.clone())
        masks.append(mask)
    sim.sync()
    sim.destroy()
    div = torch.stack([torch.nn.functional.pad(d, (0, _pitch(size) - size)) for d in divs])
    mask = torch.stack([torch.nn.functional.pad(m, (0, _pitch(size) - size)) for m in masks])
    return div.contiguous(), mask.contiguous()


def _pitch(w: int) -> int:
    return (w + 31) // 32 * 32


def make_pairs(size: int, n: int, seed: int, rtol: float = 1e-6, batch: int = 64) -> PairSet:
    div, mask = solver_snapshots(size, n, seed)
    pitch = div.shape[2]
    inv = inv_scale_of(div, mask)
    targets, rels, its = [], [], 0
    for b0 in range(0, n, batch):
        sl = slice(b0, min(n, b0 + batch))
        t, rel, it = cg_solve(div[sl].contiguous(), mask[sl].contiguous(), inv[sl].contiguous(),
                              size, size, pitch, rtol=rtol)
        targets.append(t)
        rels.append(rel)
        its = max(its, it)
    return PairSet(div, mask, inv, torch.cat(targets), torch.cat(rels), its)


def network_guess(sim, net: UNet, mask: Optional[torch.Tensor]) -> torch.Tensor:
    """The network's pressure prediction for the simulator's current system
    (dense H x W float32, in the solver's pressure units)."""
    H, W = sim.height, sim.width
    pitch = sim.divergence.stride(0)
    dfull = torch.zeros(1, H, pitch, dtype=torch.float32, device="cuda")
    dfull[0, :, :W] = sim.divergence
    m = None
    if mask is not None:
        m = torch.zeros(1, H, pitch, dtype=torch.uint8, device="cuda")
        m[0, :, :W] = mask.view(H, -1)[:, :W]
    inv = inv_scale_of(dfull[:, :, :W], m[:, :, :W] if m is not None else None)
    p = net.forward(dfull, m, inv, H, W, pitch)
    return (p[0] / inv[0]).contiguous()


def warm_start_solve(sim, net: Optional[UNet], mask: Optional[torch.Tensor], rtol: float = 1e-4,
                     check: int = 100, max_sweeps: int = 200_000_000, fallback_sweeps: int = 10,
                     time_limit_s: float = 120.0, regions: Optional[Regions] = None,
                     force: bool = False) -> dict:
    """Solve the pressure system of the simulator's last step to relative
    residual `rtol` with Jacobi sweeps, from zero (net None) or from the
    network's prediction.  Fallback rule: if the residual after
    `fallback_sweeps` sweeps from the prediction exceeds the residual after
    as many sweeps from zero, restart from zero; `force` skips the rule and
    always sweeps from the prediction.  The residual is taken over the fluid
    cells of `mask` (the obstacles the step used) with each connected
    region's mean removed; obstacle cells, whose rows the sweep updates but
    no fluid cell reads, are left out.  Labelling the regions happens before
    the clock starts.  Returns sweeps, seconds, the residual reached, whether
    the fallback fired and, with the rule, both arms' residuals after
    `fallback_sweeps` sweeps."""
    import time

    from .. import _lib as L

    H, W = sim.height, sim.width
    pitch = sim.divergence.stride(0)
    # residual over the fluid cells of the step's obstacle mask, with each
    # connected region's mean removed (the operator's null space)
    if regions is None:
        regions = Regions(mask.view(1, H, -1) if mask is not None else None, 1, H, W)
    labels, n_labels = regions.image_labels(0)

    def resid() -> float:
        return sim.residual_regions(labels, n_labels)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    used_fallback = False

    def set_pressure(p_dense: Optional[torch.Tensor]):
        pv = sim.pressure
        if p_dense is None:
            pv.zero_()
        else:
            pv.copy_(p_dense)

    r_net = r_zero = None
    if net is not None and force:
        set_pressure(network_guess(sim, net, mask))
        sweeps = 0
    elif net is not None:
        guess = network_guess(sim, net, mask)
        set_pressure(guess)
        sim.jacobi(fallback_sweeps)
        r_net = resid()
        set_pressure(None)
        sim.jacobi(fallback_sweeps)
        r_zero = resid()
        if r_net <= r_zero:
            set_pressure(guess)
            sim.jacobi(fallback_sweeps)
        else:
            used_fallback = True
        sweeps = fallback_sweeps
    else:
        set_pressure(None)
        sweeps = 0
    res = resid()
    while res > rtol and sweeps < max_sweeps and time.perf_counter() - t0 < time_limit_s:
        # residual checks every `check` sweeps, then every 5% of the sweeps so far
        k = max(check, sweeps // 20)
        sim.jacobi(k)
        sweeps += k
        res = resid()
    torch.cuda.synchronize()
    out = {"sweeps": sweeps, "seconds": time.perf_counter() - t0, "residual": res,
           "fallback": used_fallback, "converged": res <= rtol}
    if r_net is not None:
        out["residual_after_fallback_sweeps"] = {"network": r_net, "zero": r_zero}
    return out


def exact_pressure(sim, regions: Regions) -> torch.Tensor:
    """FP64 conjugate-gradient solution of the simulator's current system to
    relative residual 1e-8 (dense H x W float64, each fluid region's mean
    removed, in the solver's pressure units)."""
    H, W = sim.height, sim.width
    P = _pitch(W)
    div = torch.zeros(1, H, P, dtype=torch.float32, device="cuda")
    div[0, :, :W] = sim.divergence
    mask = torch.zeros(1, H, P, dtype=torch.uint8, device="cuda")
    mask[0, :, :W] = (~regions.fluid).to(torch.uint8)
    inv = inv_scale_of(div[:, :, :W], mask[:, :, :W])
    p, _, _ = cg_solve(div, mask, inv, H, W, P, rtol=1e-8, max_iter=200000, regions=regions,
                       as_double=True)
    return p[0].double() / float(inv[0])


def low_modes(e: torch.Tensor, kmax: int = 4) -> torch.Tensor:
    """Coefficients of a field (H x W, zero on obstacles) on the domain's
    slowest Neumann cosine modes cos(pi k (x + 1/2) / W) cos(pi l (y + 1/2) /
    H), 0 <= k, l <= kmax, without the constant: the components that plain
    Jacobi reduces slowest (their decay takes of the order of (W/pi)^2
    sweeps)."""
    H, W = e.shape
    xs = (torch.arange(W, dtype=torch.float64, device=e.device) + 0.5) / W
    ys = (torch.arange(H, dtype=torch.float64, device=e.device) + 0.5) / H
    k = torch.arange(kmax + 1, dtype=torch.float64, device=e.device)
    cx = torch.cos(math.pi * k[:, None] * xs[None, :])  # K x W
    cy = torch.cos(math.pi * k[:, None] * ys[None, :])  # K x H
    a = cy @ e.double() @ cx.T / (H * W)
    a[0, 0] = 0.0
    return a


def guess_diagnostics(sim, net: UNet, mask: Optional[torch.Tensor], regions: Regions,
                      exact: Optional[torch.Tensor] = None, kmax: int = 4) -> dict:
    """How close the network's guess is to the exact solution, overall and on
    the slowest modes, against the zero guess (whose error is the solution
    itself): rel_error = ||P(g - x)|| / ||P(x)|| and low_mode_ratio =
    ||low(P(g - x))|| / ||low(P(x))||, P removing each fluid region's mean
    and zeroing obstacles.  A warm start cuts the sweeps to a residual target
    only as far as it shrinks the low-mode error."""
    H, W = sim.height, sim.width
    if exact is None:
        exact = exact_pressure(sim, regions)
    g = network_guess(sim, net, mask).double()
    ex = regions.project(exact.view(1, H, W))[0]
    err = regions.project((g - exact).view(1, H, W))[0]
    nx = float(ex.norm())
    lx = float(low_modes(ex, kmax).norm())
    return {"rel_error": float(err.norm()) / nx if nx > 0 else 0.0,
            "low_mode_ratio": float(low_modes(err, kmax).norm()) / lx if lx > 0 else 0.0,
            "kmax": kmax}


def train(net: UNet, pairs: PairSet, steps: int, batch: int = 64, lr: float = 1e-3,
          lam: float = 1.0, seed: int = 0, log_every: int = 0) -> list:
    """Adam on random mini-batches of `pairs` (sampled with replacement)."""
    size_h, size_w = pairs.target.shape[1], pairs.target.shape[2]
    P = pairs.div.shape[2]
    if net.step_count == 0:
        net.out_scale = float(pairs.target.double().pow(2).mean().sqrt().clamp(min=1e-6))
    g = torch.Generator().manual_seed(seed)
    losses = []
    for it in range(steps):
        idx = torch.randint(0, pairs.n, (min(batch, pairs.n),), generator=g).cuda()
        losses.append(net.train_step(pairs.div[idx].contiguous(), pairs.mask[idx].contiguous(),
                                     pairs.inv_scale[idx].contiguous(),
                                     pairs.target[idx].contiguous(), size_h, size_w, P, lr=lr,
                                     lam=lam))
        if log_every and it % log_every == 0:
            print(f"step {it} loss {losses[-1]:.5g}", flush=True)
    net.check_status()
    return losses


def project_divergence(sim, regions: Regions) -> float:
    """Remove each connected fluid region's mean from the simulator's last
    divergence field, in place, and return the largest |mean| / RMS removed.

    The reference's divergence does not sum to zero over a region (the
    obstacle substitution breaks the discrete flux balance), so its pressure
    system has no solution: Jacobi then converges on the rest of the residual
    while each region's pressure drifts by a constant every sweep, and in
    FP32 the growing constant eats the precision of the solution.  The
    projected system is the solvable part; both arms of a solve-time
    comparison must use the same one."""
    H, W = sim.height, sim.width
    d = sim.divergence
    b = d.double().view(1, H, W)
    fl = regions.fluid.view(1, H, W)
    rms = float(b[fl].pow(2).mean().sqrt()) if bool(fl.any()) else 0.0
    pb = regions.project(torch.where(fl, b, torch.zeros_like(b)))
    removed = torch.where(fl, b - pb, torch.zeros_like(b))
    d.copy_(torch.where(fl, pb, b).view(H, W).float())
    return float(removed.abs().max()) / rms if rms > 0 else 0.0


def fp32_floor(sim, regions: Regions, exact: Optional[torch.Tensor] = None) -> float:
    """Relative residual of the FP64 conjugate-gradient solution of the
    simulator's current system once rounded to FP32: the lowest residual a
    solver that stores the pressure in FP32 can reach.  Leaves the pressure
    field holding that rounded solution."""
    if exact is None:
        exact = exact_pressure(sim, regions)
    sim.pressure.copy_(exact.float())
    labels, n = regions.image_labels(0)
    return sim.residual_regions(labels, n)


def evaluation_system(size: int, seed: int, steps: int = 5):
    """A simulator of the given size after `steps` steps of the large
    workload's settings, and the obstacle mask its last step used."""
    from .. import workloads as wl
    from .fluid_simulator import FluidSimulator

    sim = FluidSimulator(size, size)
    sim.iterations, sim.vorticity, sim.viscosity, sim.speed, sim.dissipation = 80, 0.35, 0.0, 5.0, 0.99
    rng = np.random.default_rng(seed)
    obst = wl.circle_obstacles(rng, 12, size, size)
    mask = None
    for _ in range(steps):
        for o in obst:
            sim.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
        mask = sim.obstacles.clone()
        sim.add_splats(wl.gauss_splats(rng, 16, size, size, 5.0))
        sim.update(1 / 60)
    return sim, mask
