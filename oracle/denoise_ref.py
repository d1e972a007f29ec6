"""CPU reference of the fluence denoiser (test infrastructure only; never imported by the package).

A plain PyTorch fp32 restatement of the U-Net in mcx_gb300/denoise.py -- same parameters, same
layer plan, same input features, same masked-L1 loss -- whose autograd gradients are the oracle
for the GPU kernels' forward, data-gradient, weight-gradient and optimiser passes.  The reference
MCX has no learned denoiser, so there is no reference-side implementation to follow; the
convolution convention (cross-correlation, zero padding 1, tap = dz*9 + dy*3 + dx over
(z, y, x) offsets -1..1) is PyTorch's conv3d on [N, C, D, H, W] tensors.
"""

from __future__ import annotations

import math

import numpy as np
import torch
import torch.nn.functional as F

LAYERS = [
    ("enc1a", 16, 16, 0), ("enc1b", 16, 16, 0),
    ("enc2a", 16, 32, 1), ("enc2b", 32, 32, 1),
    ("enc3a", 32, 64, 2), ("enc3b", 64, 64, 2),
    ("bota", 64, 128, 3), ("botb", 128, 128, 3),
    ("dec3a", 192, 64, 2), ("dec3b", 64, 64, 2),
    ("dec2a", 96, 32, 1), ("dec2b", 32, 32, 1),
    ("dec1a", 48, 16, 0), ("dec1b", 16, 16, 0),
]


def torch_weight(w: np.ndarray | torch.Tensor) -> torch.Tensor:
    """[cout, 27, cin] (tap = dz*9 + dy*3 + dx) -> conv3d's [cout, cin, kd, kh, kw]."""
    w = torch.as_tensor(w)
    cout, taps, cin = w.shape
    k = round(taps ** (1.0 / 3.0))
    return w.reshape(cout, k, k, k, cin).permute(0, 4, 1, 2, 3).contiguous()


def engine_weight(wt: torch.Tensor) -> torch.Tensor:
    """conv3d's [cout, cin, kd, kh, kw] -> [cout, 27, cin]."""
    cout, cin = wt.shape[:2]
    return wt.permute(0, 2, 3, 4, 1).reshape(cout, -1, cin)


def conv(x: torch.Tensor, w: torch.Tensor, b: torch.Tensor | None, relu: bool = True) -> torch.Tensor:
    """x [N, C, D, H, W]; w in the engine's [cout, taps, cin] order."""
    taps = w.shape[1]
    y = F.conv3d(x, torch_weight(w), b, padding=1 if taps == 27 else 0)
    return F.relu(y) if relu else y


def box_means(flux: np.ndarray, edge: tuple[int, int, int]) -> tuple[np.ndarray, np.ndarray]:
    """Means of the fluence over the in-bounds voxels of each voxel's 3x3x3 and 5x5x5
    neighbourhoods; flux [nvol, vox] in voxel order x fastest over a (d, h, w) = edge grid."""
    d, h, w = edge
    f = np.maximum(np.asarray(flux, np.float64), 0).reshape(-1, d, h, w)
    out = []
    for r in (1, 2):
        s = np.zeros_like(f)
        cnt = np.zeros((d, h, w))
        pad = np.pad(f, ((0, 0), (r, r), (r, r), (r, r)))
        one = np.pad(np.ones((d, h, w)), r)
        for dz in range(2 * r + 1):
            for dy in range(2 * r + 1):
                for dx in range(2 * r + 1):
                    s += pad[:, dz:dz + d, dy:dy + h, dx:dx + w]
                    cnt += one[dz:dz + d, dy:dy + h, dx:dx + w]
        out.append((s / cnt).reshape(f.shape[0], -1))
    return out[0], out[1]


def features(flux: np.ndarray, labels: np.ndarray, props: np.ndarray, log_photons: np.ndarray,
             edge: tuple[int, int, int]) -> tuple:
    """The 16 input channels (7 used) and residual base, restating mcxg_dn_pack on [nvol, vox]
    arrays over a (d, h, w) grid, with l0, l3, l5 = log10(m + 1e-10) of the fluence and of its
    3x3x3 and 5x5x5 in-bounds means:
      0: (l3 + 5) / 3          1: clamp(4 (l0 - l3), -4, 4)       2: clamp(4 (l5 - l3), -4, 4)
      3: 1 where the fluence is 0, else 0
      4: log10(mua) + 2        5: log10(mus (1 - g))              6: (log10(photons) - 5.5) * 2
    and the residual base l3."""
    nvol, vox = flux.shape
    lab = np.minimum(labels.astype(np.int64), props.shape[1] - 1)
    pr = np.take_along_axis(props, lab[..., None].repeat(4, -1), axis=1)        # [nvol, vox, 4]
    b3, b5 = box_means(flux, edge)
    lg = lambda a: np.log10(np.maximum(a, 0).astype(np.float32) + np.float32(1e-10)).astype(np.float32)  # noqa: E731
    l0, l3, l5 = lg(flux), lg(b3), lg(b5)
    x = np.zeros((nvol, vox, 16), np.float32)
    x[..., 0] = (l3 + 5.0) / 3.0
    x[..., 1] = np.clip(4.0 * (l0 - l3), -4.0, 4.0)
    x[..., 2] = np.clip(4.0 * (l5 - l3), -4.0, 4.0)
    x[..., 3] = (np.asarray(flux) <= 0).astype(np.float32)
    with np.errstate(divide="ignore"):
        x[..., 4] = np.where(pr[..., 0] > 0, np.log10(np.where(pr[..., 0] > 0, pr[..., 0], 1.0)) + 2.0, -2.0)
        musp = pr[..., 1] * (1.0 - pr[..., 2])
        x[..., 5] = np.where(musp > 0, np.log10(np.where(musp > 0, musp, 1.0)), -3.0)
    x[..., 6] = ((log_photons - 5.5) * 2.0)[:, None]
    return x, l3


def forward(params: dict, x0: torch.Tensor, xres: torch.Tensor, nvol: int, d: int, h: int, w: int) -> torch.Tensor:
    """Predicted log10 fluence [nvol * d * h * w] from channels-last features x0
    [nvol * d * h * w, 16] and the residual base xres; `params` maps names to tensors."""
    x = x0.reshape(nvol, d, h, w, -1).permute(0, 4, 1, 2, 3)

    def c(name, t):
        return conv(t, params[name + ".w"], params[name + ".b"])

    e1 = c("enc1b", c("enc1a", x))
    e2 = c("enc2b", c("enc2a", F.avg_pool3d(e1, 2)))
    e3 = c("enc3b", c("enc3a", F.avg_pool3d(e2, 2)))
    e4 = c("botb", c("bota", F.avg_pool3d(e3, 2)))
    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")  # noqa: E731
    d3 = c("dec3b", c("dec3a", torch.cat([up(e4), e3], 1)))
    d2 = c("dec2b", c("dec2a", torch.cat([up(d3), e2], 1)))
    d1 = c("dec1b", c("dec1a", torch.cat([up(d2), e1], 1)))
    head = torch.einsum("ncdhw,c->ndhw", d1, params["head.w"]) + params["head.b"]
    return xres + head.reshape(-1)


def loss(params: dict, x0, xres, target, valid, inv: float, nvol, d, h, w) -> torch.Tensor:
    out = forward(params, x0, xres, nvol, d, h, w)
    return ((out - target).abs() * valid).sum() * inv


def grads(params_np: dict, x0, xres, target, valid, inv, nvol, d, h, w, dtype=torch.float32):
    """(loss, output, gradients) with every parameter as a leaf tensor of `dtype`."""
    P = {k: torch.tensor(v, dtype=dtype, requires_grad=True) for k, v in params_np.items()}
    args = [torch.as_tensor(a, dtype=dtype) for a in (x0, xres, target, valid)]
    out = forward(P, args[0], args[1], nvol, d, h, w)
    L = ((out - args[2]).abs() * args[3]).sum() * inv
    L.backward()
    return float(L.detach()), out.detach(), {k: p.grad.detach().numpy() for k, p in P.items()}


def adamw(p, g, m, v, lr, b1, b2, eps, wd, step):
    """Decoupled-weight-decay Adam (Loshchilov and Hutter) in float64: returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * (wd * p + mh / (np.sqrt(vh) + eps)), m, v


def bf16(a: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even to bfloat16, returned as float32."""
    return torch.as_tensor(np.asarray(a, np.float32)).to(torch.bfloat16).float().numpy()


def he_std(cin: int, taps: int = 27) -> float:
    return math.sqrt(2.0 / (taps * cin))
