"""Seeded synthetic GUPPI RAW blocks.

Blocks are laid out as in a GUPPI RAW file (and in rawspec's host block
buffers): [channel][time][pol][re, im], one signed byte per component for
8-bit data, two little-endian bytes for 16-bit data, and one byte per complex
sample for 4-bit data (high nibble real, low nibble imaginary).  The same
bytes feed the GPU library, the FP64 oracle and the CPU baseline.
"""
from __future__ import annotations

import numpy as np


def gaussian_blocks(nblocks: int, Nc: int, Ntpb: int, Np: int = 2, sigma: float = 16.0, seed: int = 1,
                    nbits: int = 8, tone: tuple[int, float, float] | None = None, tone_nt: int = 1024) -> np.ndarray:
    """Complex Gaussian voltages, sigma per component, rounded and clipped to
    the signed nbits range; returns uint8 [nblocks, block_bytes].

    tone = (channel, fine_offset, amplitude) adds a complex exponential at
    fine frequency (tone_nt/4 + fine_offset) / tone_nt cycles per sample to
    both polarisations of that channel before quantisation."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lim = (1 << (nbits - 1))
    dtype = np.int8 if nbits == 8 else np.int16
    out = np.empty((nblocks, Nc, Ntpb, Np, 2), dtype=dtype)
    for b in range(nblocks):
        v = rng.standard_normal((Nc, Ntpb, Np, 2), dtype=np.float32) * np.float32(sigma)
        if tone is not None:
            ch, off, amp = tone
            t = np.arange(b * Ntpb, (b + 1) * Ntpb, dtype=np.float64)
            ph = 2 * np.pi * (tone_nt / 4 + off) / tone_nt * t
            v[ch, :, :, 0] += (amp * np.cos(ph)).astype(np.float32)[:, None]
            v[ch, :, :, 1] += (amp * np.sin(ph)).astype(np.float32)[:, None]
        np.rint(v, out=v)
        np.clip(v, -lim, lim - 1, out=v)
        out[b] = v.astype(dtype)
    return out.reshape(nblocks, -1).view(np.uint8)


def int4_blocks(nblocks: int, Nc: int, Ntpb: int, Np: int = 2, Nant: int = 1, seed: int = 3,
                gain_range: tuple[float, float] = (0.5, 2.0)) -> tuple[np.ndarray, np.ndarray]:
    """Packed 4-bit complex voltages: uniform in [-8, 7] per component, scaled
    by a per-antenna gain drawn from the seed before quantisation.  Returns
    (uint8 [nblocks, Nc*Ntpb*Np], gains[Nant])."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gains = rng.uniform(gain_range[0], gain_range[1], size=Nant)
    nca = Nc // Nant
    out = np.empty((nblocks, Nc, Ntpb, Np), dtype=np.uint8)
    for b in range(nblocks):
        u = rng.uniform(-8.0, 8.0, size=(Nc, Ntpb, Np, 2))
        u *= np.repeat(gains, nca)[:, None, None, None]
        q = np.clip(np.floor(u), -8, 7).astype(np.int16)
        out[b] = (((q[..., 0] & 0xF) << 4) | (q[..., 1] & 0xF)).astype(np.uint8)
    return out.reshape(nblocks, -1), gains


def weights(Nant: int, seed: int = 5, lo: float = 0.5, hi: float = 1.5) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(lo, hi, size=Nant).astype(np.float32)


def gaussian_buffer_cuda(index: int, nblocks: int, Nc: int, Ntpb: int, Np: int = 2, sigma: float = 20.0,
                         seed: int = 1, device: int = 0) -> np.ndarray:
    """Blocks index*nblocks ... index*nblocks + nblocks - 1 of a seeded stream
    of complex Gaussian 8-bit voltages (sigma per component, rounded half to
    even and clipped to [-128, 127]), drawn on the GPU with torch's
    counter-based generator, one seed per block, so that any process on the
    same GPU model and torch version draws the same bytes.  For inputs too
    large to generate on the host (the production shape over many buffers).
    Returns uint8 [nblocks, block_bytes] in host memory."""
    import torch
    dev = torch.device("cuda", device)
    out = np.empty((nblocks, Nc * Ntpb * Np * 2), dtype=np.uint8)
    g = torch.Generator(device=dev)
    for j in range(nblocks):
        g.manual_seed(seed * 1000003 + index * nblocks + j)
        v = torch.randn((Nc, Ntpb, Np, 2), generator=g, device=dev, dtype=torch.float32) * sigma
        v = torch.round(v).clamp_(-128, 127).to(torch.int8)
        out[j] = v.view(torch.uint8).reshape(-1).cpu().numpy()
    return out
