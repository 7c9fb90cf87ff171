"""Local-window additive Gaussian renderer (python/wgnet/render.py), with its forward and backward on
hand-written CUDA kernels.

Layout as in the reference: one slot per 2x2-pixel cell of the 70x70 grid (35x35 = 1225 slots),
6 activated parameters per slot `(dx, dz, log_sx, log_sz, angle, amp)`, each slot drawn in the
25x25 pixel window around its anchor. `render_residual` is differentiable through
`torch.autograd` (the backward is the CUDA VJP kernel). Parameter activation/clamping keep the
reference's expressions (they define the parametrisation); the metrics (MAE, RMSE, SSIM) are
written here as a separable-window SSIM.
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


_WINDOWS: dict[str, tuple[torch.Tensor, torch.Tensor, torch.Tensor]] = {}


def slot_windows(device: torch.device | str = "cpu") -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """The pixels each slot draws (render.py:44-61): `(flat [N_SLOTS, 625] int64, centres
    [N_SLOTS, 625, 2] f32, valid [N_SLOTS, 625] f32)`. Slot s = 35 iz + ix sits on pixel
    (2 iz, 2 ix); window entry k covers pixel (2 iz + k // 25 - 12, 2 ix + k % 25 - 12), whose centre
    is at index + 0.5. Pixels outside the 70 x 70 grid get the spare index 4900 and valid 0.
    The CUDA kernels derive the same windows arithmetically; these tables serve callers that
    scatter per-window values themselves."""
    key = str(device)
    hit = _WINDOWS.get(key)
    if hit is not None:
        return hit
    slot = torch.arange(N_SLOTS, device=device)
    k = torch.arange(WIN_SIDE * WIN_SIDE, device=device)
    rows = 2 * torch.div(slot, SLOT_SIDE, rounding_mode="floor")[:, None] + (
        torch.div(k, WIN_SIDE, rounding_mode="floor") - WINDOW)[None, :]
    cols = 2 * torch.remainder(slot, SLOT_SIDE)[:, None] + (torch.remainder(k, WIN_SIDE) - WINDOW)[None, :]
    inside = (rows >= 0) & (rows < GRID) & (cols >= 0) & (cols < GRID)
    flat = torch.where(inside, rows * GRID + cols, torch.full_like(rows, GRID * GRID))
    centres = torch.stack([cols.to(torch.float32) + 0.5, rows.to(torch.float32) + 0.5], dim=-1)
    out = (flat, centres, inside.to(torch.float32))
    _WINDOWS[key] = out
    return out


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


# SSIM constants (Wang et al. 2004): an 11-tap Gaussian window of standard deviation 1.5 pixels,
# stabilisers (0.01 L)^2 and (0.03 L)^2 for a dynamic range L = 1 of the normalised fields.
SSIM_TAPS = 11
SSIM_SIGMA = 1.5
SSIM_C1 = 0.01**2
SSIM_C2 = 0.03**2


def _ssim_taps(device, dtype) -> torch.Tensor:
    """Normalised 1-D Gaussian; the 2-D SSIM window is its outer product with itself."""
    r = torch.linspace(-(SSIM_TAPS // 2), SSIM_TAPS // 2, SSIM_TAPS, device=device, dtype=torch.float64)
    g = torch.exp(-(r * r) / (2.0 * SSIM_SIGMA * SSIM_SIGMA))
    return (g / g.sum()).to(dtype)


def _local_means(stack: torch.Tensor, taps: torch.Tensor) -> torch.Tensor:
    """Windowed means of every channel of `[B, C, H, W]` over the valid (unpadded) region, as two
    1-D passes (rows, then columns) of one grouped convolution each."""
    c = stack.shape[1]
    kx = taps.view(1, 1, 1, -1).expand(c, 1, 1, SSIM_TAPS)
    kz = taps.view(1, 1, -1, 1).expand(c, 1, SSIM_TAPS, 1)
    return F.conv2d(F.conv2d(stack, kx, groups=c), kz, groups=c)


def ssim(pred_km: torch.Tensor, target_km: torch.Tensor) -> torch.Tensor:
    """Per-sample mean SSIM `[B]` of two velocity fields after the OpenFWI normalisation
    (v - 1.5) / 3 km/s (render.py:123-137 defines the metric): the five local moments of the pair
    come from one separable Gaussian filtering of the stacked channels (x, y, x^2, y^2, x y)."""
    x = (pred_km - V_MIN_KM) / (V_MAX_KM - V_MIN_KM)
    y = (target_km - V_MIN_KM) / (V_MAX_KM - V_MIN_KM)
    moments = _local_means(torch.stack([x, y, x * x, y * y, x * y], dim=1), _ssim_taps(x.device, x.dtype))
    mx, my, exx, eyy, exy = moments.unbind(dim=1)
    mxy = mx * my
    var_sum = (exx - mx * mx) + (eyy - my * my)
    cov = exy - mxy
    index = ((2.0 * mxy + SSIM_C1) * (2.0 * cov + SSIM_C2)) / ((mx * mx + my * my + SSIM_C1) * (var_sum + SSIM_C2))
    return index.flatten(1).mean(dim=1)


@torch.no_grad()
def field_metrics(pred_km: torch.Tensor, target_km: torch.Tensor) -> dict[str, torch.Tensor]:
    """Per-sample `[B]` velocity errors (render.py:140-152 defines the set): mean absolute and root
    mean square error in m/s, SSIM, and the OpenFWI-normalised MAE and MSE (errors in units of
    1500 m/s)."""
    err_mps = ((pred_km - target_km) * 1000.0).flatten(1)
    mae = err_mps.abs().mean(dim=1)
    mse = (err_mps * err_mps).mean(dim=1)
    return {"mae_mps": mae, "rmse_mps": torch.sqrt(mse), "ssim": ssim(pred_km, target_km), "mae_norm": mae / 1500.0,
            "mse_norm": mse / (1500.0 * 1500.0)}
