"""Local-window additive Gaussian renderer (python/wgnet/render.py), with its forward and backward on
hand-written CUDA kernels.

Layout as in the reference: one slot per 2x2-pixel cell of the 70x70 grid (35x35 = 1225 slots),
6 activated parameters per slot `(dx, dz, log_sx, log_sz, angle, amp)`, each slot drawn in the
25x25 pixel window around its anchor. `render_residual` is differentiable through
`torch.autograd` (the backward is the CUDA VJP kernel). Parameter activation/clamping and the
metrics (MAE, RMSE, SSIM) are small torch expressions, as in the reference.
"""

from __future__ import annotations

import math

import torch
import torch.nn.functional as F

from . import _lib
from ._lib import check, ptr

GRID = 70
SLOT_SIDE = 35
N_SLOTS = SLOT_SIDE * SLOT_SIDE
WINDOW = 12
WIN_SIDE = 2 * WINDOW + 1
OFFSET_MAX = 2.0
SIGMA_MIN = 0.5
SIGMA_MAX = 6.0
AMP_MAX = 1.0
ACTIVE_AMP_KM = 0.05
N_GAUSS_PARAMS = 6
V_MIN_KM, V_MAX_KM = 1.5, 4.5


def slot_anchors(device: torch.device | str = "cpu") -> torch.Tensor:
    """`[N_SLOTS, 2]` anchor positions `(x, z)` in pixel-edge coordinates (render.py:34-38)."""
    i = torch.arange(SLOT_SIDE, device=device, dtype=torch.float32)
    gz, gx = torch.meshgrid(2.0 * i + 1.0, 2.0 * i + 1.0, indexing="ij")
    return torch.stack([gx.reshape(-1), gz.reshape(-1)], dim=-1)


def activate_gaussians(raw: torch.Tensor) -> torch.Tensor:
    """Unconstrained `[..., 6]` -> bounded physical parameters (render.py:64-73)."""
    dx = OFFSET_MAX * torch.tanh(raw[..., 0])
    dz = OFFSET_MAX * torch.tanh(raw[..., 1])
    log_range = math.log(SIGMA_MAX) - math.log(SIGMA_MIN)
    log_sx = math.log(SIGMA_MIN) + log_range * torch.sigmoid(raw[..., 2])
    log_sz = math.log(SIGMA_MIN) + log_range * torch.sigmoid(raw[..., 3])
    angle = (math.pi / 2.0) * torch.tanh(raw[..., 4])
    amp = AMP_MAX * torch.tanh(raw[..., 5])
    return torch.stack([dx, dz, log_sx, log_sz, angle, amp], dim=-1)


def clamp_gaussians(params: torch.Tensor) -> torch.Tensor:
    """Project activated parameters back into their bounds (render.py:76-83)."""
    out = params.clone()
    out[..., 0:2] = out[..., 0:2].clamp(-OFFSET_MAX, OFFSET_MAX)
    out[..., 2:4] = out[..., 2:4].clamp(math.log(SIGMA_MIN), math.log(SIGMA_MAX))
    out[..., 4] = out[..., 4].clamp(-math.pi / 2.0, math.pi / 2.0)
    out[..., 5] = out[..., 5].clamp(-AMP_MAX, AMP_MAX)
    return out


def _stream(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor) -> torch.Tensor:
        p = params.detach().float().contiguous()
        b = p.shape[0]
        out = torch.empty((b, GRID, GRID), device=p.device, dtype=torch.float32)
        with torch.cuda.device(p.device):
            check(_lib.load().wg_render_fwd_dev(ptr(p), b, ptr(out), _stream(p)), "render_residual")
        ctx.save_for_backward(p)
        return out

    @staticmethod
    def backward(ctx, cot: torch.Tensor):
        (p,) = ctx.saved_tensors
        c = cot.detach().float().contiguous()
        g = torch.empty_like(p)
        with torch.cuda.device(p.device):
            check(_lib.load().wg_render_bwd_dev(ptr(p), ptr(c), p.shape[0], ptr(g), _stream(p)), "render_residual")
        return g


def render_residual(params: torch.Tensor) -> torch.Tensor:
    """Render activated slot parameters `[B, N_SLOTS, 6]` to a residual field `[B, 70, 70]` in km/s
    (render.py:86-109). CPU tensors are moved to the current CUDA device for the kernels and the
    result is returned on the input's device."""
    if params.ndim != 3 or params.shape[1] != N_SLOTS or params.shape[2] != N_GAUSS_PARAMS:
        raise ValueError(f"params must be [B, {N_SLOTS}, {N_GAUSS_PARAMS}]")
    if params.is_cuda:
        return _Render.apply(params).to(params.dtype)
    out = _Render.apply(params.to("cuda", torch.float32))
    return out.to(device=params.device, dtype=params.dtype)


def _gaussian_window(size: int = 11, sigma: float = 1.5, device="cpu") -> torch.Tensor:
    x = torch.arange(size, device=device, dtype=torch.float32) - (size - 1) / 2.0
    g = torch.exp(-0.5 * (x / sigma) ** 2)
    g = g / g.sum()
    return (g[:, None] * g[None, :]).view(1, 1, size, size)


def ssim(pred_km: torch.Tensor, target_km: torch.Tensor) -> torch.Tensor:
    """Per-sample SSIM `[B]` on `(v - 1.5) / 3.0`, 11x11 Gaussian window (render.py:123-137)."""
    scale = V_MAX_KM - V_MIN_KM
    x = ((pred_km - V_MIN_KM) / scale).unsqueeze(1)
    y = ((target_km - V_MIN_KM) / scale).unsqueeze(1)
    w = _gaussian_window(device=pred_km.device).to(x.dtype)
    c1, c2 = 0.01**2, 0.03**2
    mu_x = F.conv2d(x, w)
    mu_y = F.conv2d(y, w)
    sxx = F.conv2d(x * x, w) - mu_x**2
    syy = F.conv2d(y * y, w) - mu_y**2
    sxy = F.conv2d(x * y, w) - mu_x * mu_y
    num = (2 * mu_x * mu_y + c1) * (2 * sxy + c2)
    den = (mu_x**2 + mu_y**2 + c1) * (sxx + syy + c2)
    return (num / den).mean(dim=(1, 2, 3))


@torch.no_grad()
def field_metrics(pred_km: torch.Tensor, target_km: torch.Tensor) -> dict[str, torch.Tensor]:
    """Per-sample `[B]` MAE and RMSE in m/s, SSIM, OpenFWI-normalized MAE / MSE (render.py:140-152)."""
    err = (pred_km - target_km) * 1000.0
    mae = err.abs().mean(dim=(1, 2))
    mse = err.square().mean(dim=(1, 2))
    return {"mae_mps": mae, "rmse_mps": mse.sqrt(), "ssim": ssim(pred_km, target_km), "mae_norm": mae / 1500.0,
            "mse_norm": mse / 1500.0**2}
