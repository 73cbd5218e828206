"""Seeded synthetic microscopy stacks: the stand-in for real data.

Constant background 100 plus K isotropic Gaussian blobs (sigma ~ U[2,6] px,
peak ~ U[500,3000], uniform centres), Poisson-sampled, clipped to the pixel
type's range.  Blob parameters come from numpy's seeded generator, so they
are identical on every machine; the Poisson draw uses torch's generator on
the target device.
"""
from __future__ import annotations

import numpy as np
import torch

_RANGE = {torch.uint8: 255.0, torch.int8: 127.0, torch.uint16: 65535.0, torch.int16: 32767.0}


def blobs(shape, n_blobs: int, seed: int, dtype=torch.uint16, device="cuda", noise_sigma: float = 0.0,
          poisson: bool = True, scale_to_dtype: bool = False, chunk: int = 256) -> torch.Tensor:
    """shape: (depth, height, width) or (height, width)."""
    shape = tuple(int(v) for v in shape)
    rng = np.random.default_rng(seed)
    nd = len(shape)
    centres = np.stack([rng.uniform(0, s, n_blobs) for s in shape], axis=1)
    sig = rng.uniform(2.0, 6.0, n_blobs)
    peak = rng.uniform(500.0, 3000.0, n_blobs)
    img = torch.full(shape, 100.0, dtype=torch.float32, device=device)
    R = int(np.ceil(3 * 6.0))
    ax = torch.arange(-R, R + 1, device=device, dtype=torch.float32)
    grids = torch.meshgrid(*([ax] * nd), indexing="ij")
    off = torch.stack([g.reshape(-1) for g in grids], 1)  # (M, nd)
    r2 = (off ** 2).sum(1)
    flat = img.view(-1)
    strides = torch.tensor([int(np.prod(shape[i + 1:])) for i in range(nd)], device=device)
    dims = torch.tensor(shape, device=device)
    for b0 in range(0, n_blobs, chunk):
        c = torch.tensor(centres[b0:b0 + chunk], device=device, dtype=torch.float32)
        s = torch.tensor(sig[b0:b0 + chunk], device=device, dtype=torch.float32)
        p = torch.tensor(peak[b0:b0 + chunk], device=device, dtype=torch.float32)
        base = torch.floor(c).long()  # (B, nd)
        pos = base[:, None, :] + off[None, :, :].long()  # (B, M, nd)
        d = pos.float() + 0.5 - c[:, None, :]
        val = p[:, None] * torch.exp(-(d ** 2).sum(2) / (2 * s[:, None] ** 2))
        val = val * (r2[None, :] <= (3 * s[:, None]) ** 2 + 1e-6)
        ok = ((pos >= 0) & (pos < dims)).all(2)
        idx = (pos * strides).sum(2)
        flat.index_put_((idx[ok],), val[ok], accumulate=True)
    if poisson:
        g = torch.Generator(device=device)
        g.manual_seed(seed)
        img = torch.poisson(img, generator=g)
    if noise_sigma:
        g2 = torch.Generator(device=device)
        g2.manual_seed(seed + 1)
        img = img + noise_sigma * torch.randn(img.shape, generator=g2, device=device)
    if dtype == torch.float32:
        return img.contiguous()
    hi = _RANGE[dtype]
    if scale_to_dtype:
        img = img * (hi / 3100.0)
    lo = -hi - 1 if dtype in (torch.int8, torch.int16) else 0.0
    return img.clamp_(lo, hi).to(dtype).contiguous()


def mask_of(img: torch.Tensor, threshold: float = 400.0) -> torch.Tensor:
    """Binary uint8 mask, 1 where img > threshold (greater_constant_3d_x.cl:45-51)."""
    return (img.float() > threshold).to(torch.uint8)
