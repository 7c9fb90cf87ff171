"""Learned update network for refinement (no reference counterpart: WGNet's refine(),
python/wgnet/refine.py:41-169, is plain projected L-BFGS).

`UpdateNet` maps (current 70x70 velocity in km/s, the exact misfit gradient, the band index) to a
proposed model update in km/s. It is a dilated residual convolution network, ~0.45 M parameters:

    features (8 channels: v - 3, g / rms(g), one-hot band x 4, depth, 0)
    conv3x3 8 -> 64, ReLU
    6 residual blocks, dilations 1, 2, 4, 8, 4, 2:  h = h + conv3x3_d1(ReLU(conv3x3_d(h)))
    conv3x3 64 -> 1 (x 0.25 km/s)

Weights are BF16 with FP32 master copies; every convolution runs as a tensor-core GEMM
(`wg_gemm_bf16_dev`, FP32 accumulation) on im2col columns, forward, data gradient and weight
gradient alike; the glue (im2col/col2im, ReLU, residual adds, features, loss, Adam) is the
library's own kernels. PyTorch only holds the buffers.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check

CIN = 8
CH = 64
DILATIONS = (1, 2, 4, 8, 4, 2)
OUT_SCALE = 0.25
BANDS = (6.0, 9.0, 12.0, None)


def band_index(band_hz) -> int:
    return BANDS.index(band_hz) if band_hz in BANDS else 3


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class Layer:
    name: str
    cin: int
    n: int      # GEMM N (output channels, padded to 64)
    kp: int     # GEMM K (9 cin padded to 64)
    dil: int
    w32: object
    m1: object
    m2: object
    w: object   # bf16 [n][kp]
    wt: object  # bf16 [kp][n]


class UpdateNet:
    def __init__(self, seed: int = 0, device=None):
        import torch

        self._lib = _lib.load()
        self.device = torch.device(device or "cuda")
        g = np.random.default_rng(seed)
        self.layers: list[Layer] = []
        self._add("in", CIN, CH, 1, g, std=math.sqrt(2.0 / (9 * CIN)))
        for i, d in enumerate(DILATIONS):
            self._add(f"b{i}a", CH, CH, d, g, std=math.sqrt(2.0 / (9 * CH)))
            self._add(f"b{i}b", CH, CH, 1, g, std=0.1 * math.sqrt(2.0 / (9 * CH)))
        self._add("out", CH, CH, 1, g, std=1e-3, out_channels=1)
        self.step = 0
        self._bufs = {}
        self._status = torch.zeros(4, device=self.device, dtype=torch.int32)
        self._sync_bf16()

    # -- parameters ----------------------------------------------------------------------------
    def _add(self, name, cin, n, dil, g, std, out_channels=None):
        import torch

        k = 9 * cin
        kp = -(-k // 64) * 64
        w = np.zeros((n, kp), np.float32)
        rows = out_channels or n
        w[:rows, :k] = g.normal(0.0, std, (rows, k)).astype(np.float32)
        dev = self.device
        t = torch.from_numpy(w).to(dev)
        self.layers.append(Layer(name, cin, n, kp, dil, t, torch.zeros_like(t), torch.zeros_like(t),
                                 torch.empty((n, kp), device=dev, dtype=torch.bfloat16),
                                 torch.empty((kp, n), device=dev, dtype=torch.bfloat16)))

    def _sync_bf16(self):
        for L in self.layers:
            check(self._lib.wg_pc_adam(None, 0, L.n, L.kp, _p(L.w32), _p(L.m1), _p(L.m2), 0.0, 0.0, 0.0, 0.0, 0,
                                       _p(L.w), _p(L.wt), _stream()), "adam")

    @property
    def parameters(self) -> int:
        total = 0
        for L in self.layers:
            rows = 1 if L.name == "out" else L.n
            total += rows * 9 * L.cin
        return total

    def state_dict(self) -> dict:
        return {L.name: L.w32.cpu().numpy() for L in self.layers} | {"step": np.array(self.step)}

    def load_state_dict(self, d: dict) -> None:
        import torch

        for L in self.layers:
            L.w32.copy_(torch.from_numpy(np.asarray(d[L.name], np.float32)))
            L.m1.zero_()
            L.m2.zero_()
        self.step = int(d.get("step", 0))
        self._sync_bf16()

    def save(self, path) -> None:
        np.savez(path, **self.state_dict())

    @classmethod
    def load(cls, path, device=None) -> "UpdateNet":
        net = cls(device=device)
        with np.load(path) as d:
            net.load_state_dict({k: d[k] for k in d.files})
        return net

    # -- building blocks ------------------------------------------------------------------------
    def _buf(self, key, shape, dtype):
        import torch

        b = self._bufs.get(key)
        if b is None or tuple(b.shape) != tuple(shape) or b.dtype != dtype:
            b = torch.empty(shape, device=self.device, dtype=dtype)
            self._bufs[key] = b
        return b

    def _conv(self, L: Layer, x_bf16, B, H, W, out):
        import torch

        M = B * H * W
        col = self._buf(f"col{L.kp}", (M, L.kp), torch.bfloat16)
        check(self._lib.wg_pc_im2col(_p(x_bf16), B, H, W, L.cin, L.dil, L.kp, _p(col), _stream()), "im2col")
        check(self._lib.wg_gemm_bf16_dev(_p(col), _p(L.w), _p(out), M, L.n, L.kp, 1, _p(self._status), _stream()),
              "gemm")
        return out

    def _backward_conv(self, L: Layer, x_bf16, dy, B, H, W, splits, need_dx, dx=None, accumulate=0):
        """Weight gradient partials of L (returned) and, if need_dx, dx (+)= the data gradient."""
        import torch

        M = B * H * W
        dy16 = self._buf("dy16", (M, L.n), torch.bfloat16)
        check(self._lib.wg_pc_cast_bf16(_p(dy), M, L.n, L.n, 0, _p(dy16), _stream()))
        col = self._buf(f"col{L.kp}", (M, L.kp), torch.bfloat16)
        check(self._lib.wg_pc_im2col(_p(x_bf16), B, H, W, L.cin, L.dil, L.kp, _p(col), _stream()))
        colT = self._buf(f"colT{L.kp}", (L.kp, M), torch.bfloat16)
        check(self._lib.wg_pc_transpose_bf16(_p(col), M, L.kp, _p(colT), _stream()))
        dyT = self._buf("dyT", (L.n, M), torch.bfloat16)
        check(self._lib.wg_pc_transpose_bf16(_p(dy16), M, L.n, _p(dyT), _stream()))
        kt = M // 64
        per = -(-kt // splits)
        nz = -(-kt // per)
        part = torch.empty((nz, L.kp, L.n), device=self.device, dtype=torch.float32)
        check(self._lib.wg_gemm_bf16_dev(_p(colT), _p(dyT), _p(part), L.kp, L.n, M, splits, _p(self._status),
                                         _stream()), "gemm wgrad")
        if need_dx:
            dcol = self._buf(f"dcol{L.kp}", (M, L.kp), torch.float32)
            check(self._lib.wg_gemm_bf16_dev(_p(dy16), _p(L.wt), _p(dcol), M, L.kp, L.n, 1, _p(self._status),
                                             _stream()), "gemm dgrad")
            check(self._lib.wg_pc_col2im(_p(dcol), B, H, W, L.cin, L.dil, L.kp, _p(dx), accumulate, _stream()))
        return part

    # -- forward / training -----------------------------------------------------------------------
    def forward(self, vel_km, grad, band, keep: bool = False):
        """`vel_km`, `grad`: [B, H, W] float32 CUDA tensors; `band`: [B] int32 CUDA tensor of band
        indices (0..3 for 6, 9, 12 Hz and the full band). Returns the proposed update [B, H, W]
        (km/s)."""
        import torch

        if not hasattr(self, "_bufs"):
            self._bufs = {}
            self._status = torch.zeros(4, device=self.device, dtype=torch.int32)
        B, H, W = vel_km.shape
        M = B * H * W
        rms = self._buf("rms", (B,), torch.float32)
        x0 = torch.empty((M, CIN), device=self.device, dtype=torch.bfloat16)
        check(self._lib.wg_pc_features(_p(vel_km.contiguous()), _p(grad.contiguous()), _p(band.contiguous()), B, H,
                                       W, _p(rms), _p(x0), _stream()), "features")
        saved = {"x0": x0, "shape": (B, H, W)}
        L = self.layers[0]
        y = self._buf("y", (M, CH), torch.float32)
        self._conv(L, x0, B, H, W, y)
        h16 = torch.empty((M, CH), device=self.device, dtype=torch.bfloat16)
        check(self._lib.wg_pc_cast_bf16(_p(y), M, CH, CH, 1, _p(h16), _stream()))
        h = torch.empty((M, CH), device=self.device, dtype=torch.float32)
        check(self._lib.wg_pc_relu_grad(_p(y), _p(h16), M * CH, _p(h), _stream()))
        saved["h0"] = h16
        blocks = []
        for i in range(len(DILATIONS)):
            La, Lb = self.layers[1 + 2 * i], self.layers[2 + 2 * i]
            self._conv(La, h16, B, H, W, y)
            a16 = torch.empty((M, CH), device=self.device, dtype=torch.bfloat16)
            check(self._lib.wg_pc_cast_bf16(_p(y), M, CH, CH, 1, _p(a16), _stream()))
            self._conv(Lb, a16, B, H, W, y)
            hn = torch.empty((M, CH), device=self.device, dtype=torch.float32)
            hn16 = torch.empty((M, CH), device=self.device, dtype=torch.bfloat16)
            check(self._lib.wg_pc_add(_p(h), _p(y), M * CH, _p(hn), _p(hn16), _stream()))
            blocks.append((h16, a16, h))
            h, h16 = hn, hn16
        saved["blocks"] = blocks
        saved["hlast"] = h16
        saved["hlast32"] = h
        out = torch.empty((M, CH), device=self.device, dtype=torch.float32)
        self._conv(self.layers[-1], h16, B, H, W, out)
        if keep:
            self._saved = saved
            self._out = out
            self.last_activations = saved
        return (out[:, 0] * OUT_SCALE).view(B, H, W)

    def train_step(self, vel_km, grad, band, target_km, lr: float = 1e-3, splits: int = 64) -> float:
        """One Adam step on the mean squared error between the proposed update and `target_km`
        ([B, H, W], km/s). B must be a multiple of 16 (the weight-gradient reduction runs over
        B H W rows in tiles of 64). Returns the loss."""
        import torch

        self.forward(vel_km, grad, band, keep=True)
        s = self._saved
        B, H, W = s["shape"]
        M = B * H * W
        out = self._out
        dout = torch.zeros((M, CH), device=self.device, dtype=torch.float32)
        loss = torch.zeros(1, device=self.device, dtype=torch.float64)
        check(self._lib.wg_pc_mse(_p(out), CH, _p(target_km.contiguous()), OUT_SCALE, M, _p(loss), _p(dout),
                                  _stream()), "mse")
        parts = {}
        dh = torch.empty((M, CH), device=self.device, dtype=torch.float32)
        parts["out"] = self._backward_conv(self.layers[-1], s["hlast"], dout, B, H, W, splits, True, dh, 0)
        tmp = torch.empty((M, CH), device=self.device, dtype=torch.float32)
        for i in reversed(range(len(DILATIONS))):
            La, Lb = self.layers[1 + 2 * i], self.layers[2 + 2 * i]
            h16, a16, _ = s["blocks"][i]
            da = torch.empty((M, CH), device=self.device, dtype=torch.float32)
            parts[Lb.name] = self._backward_conv(Lb, a16, dh, B, H, W, splits, True, da, 0)
            check(self._lib.wg_pc_relu_grad(_p(da), _p(a16), M * CH, _p(tmp), _stream()))
            parts[La.name] = self._backward_conv(La, h16, tmp, B, H, W, splits, True, dh, 1)
        check(self._lib.wg_pc_relu_grad(_p(dh), _p(s["h0"]), M * CH, _p(tmp), _stream()))
        parts["in"] = self._backward_conv(self.layers[0], s["x0"], tmp, B, H, W, splits, False)
        self.step += 1
        for L in self.layers:
            p = parts[L.name]
            check(self._lib.wg_pc_adam(_p(p), p.shape[0], L.n, L.kp, _p(L.w32), _p(L.m1), _p(L.m2), float(lr), 0.9,
                                       0.999, 1e-8, self.step, _p(L.w), _p(L.wt), _stream()), "adam")
        self._last_parts = parts
        self._saved = None
        self.last_activations = None
        return float(loss.item())

    def status(self) -> int:
        """Device status word of the GEMM pipeline (non-zero after a timed-out wait)."""
        return int(self._status[0].item())

    def weight_gradients(self) -> dict:
        """{layer: dL/dW [n][kp]} of the last train_step (for tests)."""
        return {k: p.sum(0).t().contiguous() for k, p in self._last_parts.items()}


__all__ = ["UpdateNet", "BANDS", "band_index", "DILATIONS", "OUT_SCALE"]
