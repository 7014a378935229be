"""Seeded synthetic frame pairs for the parity tests and the benchmark.

No dataset is available offline, so these stand in for real video with the shapes and value
distributions of the benchmark configurations:

* ``rgb24_pair``       -- 8-bit RGB: per channel a sum of 8 sinusoidal gratings (orientation
                          U[0, pi), period U[4, 64] px, amplitude U[10, 40]) plus U[-8, 8] noise,
                          centred at 128, clipped and rounded; distorted = reference + N(0, 4).
* ``yuv420p10_frames`` -- 10-bit 4:2:0 limited-range Y'CbCr built from the same grating model
                          (luma x4 for 10 bits, chroma at half resolution), with a per-frame phase
                          drift of 0.05 rad; distortions are 8x8 block-DCT quantisation (step
                          U[4, 32], chroma step x2) or a Gaussian blur (sigma U[0.5, 2]) followed by
                          Gaussian noise (sigma U[1, 6]).
* ``yuv420p10_to_rgb`` -- the BT.709 conversion used to feed RGB planes to the scorers: limited ->
                          full range, bilinear chroma upsampling with MPEG-2 (left) siting, BT.709
                          matrix, gamma-encoded R'G'B' in [0, 1].

Scalar draws come from numpy's seeded generator (identical on every host); per-pixel noise comes
from a torch generator on the requested device, so CPU and GPU draws differ. Every consumer that
compares two implementations hands both the same arrays.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _gratings(h: int, w: int, rs: np.random.Generator, n: int, amp_scale: float, phase: float,
              device, out: torch.Tensor | None = None) -> torch.Tensor:
    """Sum of n sinusoidal gratings evaluated with separable outer products (float64)."""
    xs = torch.arange(w, device=device, dtype=torch.float64)
    ys = torch.arange(h, device=device, dtype=torch.float64)
    acc = torch.zeros((h, w), device=device, dtype=torch.float64) if out is None else out
    for _ in range(n):
        theta = rs.uniform(0.0, math.pi)
        period = rs.uniform(4.0, 64.0)
        amp = rs.uniform(10.0, 40.0) * amp_scale
        phi = rs.uniform(0.0, 2 * math.pi) + phase
        k = 2 * math.pi / period
        ax = k * math.cos(theta) * xs
        by = k * math.sin(theta) * ys + phi
        acc += amp * (torch.outer(torch.cos(by), torch.sin(ax)) + torch.outer(torch.sin(by), torch.cos(ax)))
    return acc


def rgb24_pair(h: int = 256, w: int = 256, seed: int = 1, device="cpu"):
    """One 8-bit RGB reference/distorted pair, each a (3, h, w) uint8 tensor."""
    rs = np.random.default_rng(seed)
    gen = torch.Generator(device=device).manual_seed(seed)
    ref = torch.empty((3, h, w), dtype=torch.uint8, device=device)
    dist = torch.empty_like(ref)
    for c in range(3):
        v = _gratings(h, w, rs, 8, 1.0, 0.0, device)
        v += (torch.rand((h, w), generator=gen, device=device, dtype=torch.float64) * 16.0 - 8.0)
        r = torch.clamp(torch.round(v + 128.0), 0, 255)
        ref[c] = r.to(torch.uint8)
        d = torch.clamp(torch.round(r + 4.0 * torch.randn((h, w), generator=gen, device=device, dtype=torch.float64)),
                        0, 255)
        dist[c] = d.to(torch.uint8)
    return ref, dist


# ------------------------------------------------------------------------------------------
# YUV 4:2:0, 10-bit

def _dct_matrix(n: int = 8, device="cpu") -> torch.Tensor:
    k = torch.arange(n, dtype=torch.float64, device=device)
    m = torch.cos(math.pi * (2 * k[None, :] + 1) * k[:, None] / (2 * n)) * math.sqrt(2.0 / n)
    m[0] /= math.sqrt(2.0)
    return m  # orthonormal DCT-II rows


def block_dct_quantise(plane: torch.Tensor, step: float, lo: int, hi: int) -> torch.Tensor:
    """8x8 block DCT, uniform quantisation of every coefficient with `step`, inverse DCT,
    rounding and clipping to [lo, hi]. Edges are padded by replication to a multiple of 8."""
    h, w = plane.shape
    ph, pw = (-h) % 8, (-w) % 8
    x = plane.to(torch.float64)
    if ph or pw:
        x = torch.nn.functional.pad(x[None, None], (0, pw, 0, ph), mode="replicate")[0, 0]
    H, W = x.shape
    D = _dct_matrix(8, x.device)
    blocks = x.reshape(H // 8, 8, W // 8, 8).permute(0, 2, 1, 3)
    coef = D @ blocks @ D.T
    coef = torch.round(coef / step) * step
    rec = (D.T @ coef @ D).permute(0, 2, 1, 3).reshape(H, W)[:h, :w]
    return torch.clamp(torch.round(rec), lo, hi).to(torch.int32)


def gaussian_blur_noise(plane: torch.Tensor, sigma: float, noise_sigma: float, lo: int, hi: int,
                        gen: torch.Generator) -> torch.Tensor:
    """Separable Gaussian blur (radius ceil(3 sigma), edge replication) then N(0, noise_sigma)."""
    x = plane.to(torch.float64)[None, None]
    r = max(1, int(math.ceil(3 * sigma)))
    t = torch.arange(-r, r + 1, dtype=torch.float64, device=x.device)
    k = torch.exp(-t * t / (2 * sigma * sigma))
    k /= k.sum()
    x = torch.nn.functional.pad(x, (r, r, 0, 0), mode="replicate")
    x = torch.nn.functional.conv2d(x, k.view(1, 1, 1, -1))
    x = torch.nn.functional.pad(x, (0, 0, r, r), mode="replicate")
    x = torch.nn.functional.conv2d(x, k.view(1, 1, -1, 1))[0, 0]
    x = x + noise_sigma * torch.randn(x.shape, generator=gen, device=x.device, dtype=torch.float64)
    return torch.clamp(torch.round(x), lo, hi).to(torch.int32)


def yuv420p10_source(h: int, w: int, t: int, seed: int, device="cpu"):
    """Reference frame t of a sequence: (Y, Cb, Cr) int32 tensors, limited range."""
    rs = np.random.default_rng(seed)  # same gratings for every frame; only the phase drifts
    gen = torch.Generator(device=device).manual_seed(seed * 100003 + t)
    phase = 0.05 * t
    y = _gratings(h, w, rs, 8, 4.0, phase, device)
    y += torch.rand((h, w), generator=gen, device=device, dtype=torch.float64) * 64.0 - 32.0
    Y = torch.clamp(torch.round(y + 502.0), 64, 940).to(torch.int32)
    ch, cw = (h + 1) // 2, (w + 1) // 2
    out = [Y]
    for _ in range(2):
        c = _gratings(ch, cw, rs, 8, 2.0, phase, device)
        c += torch.rand((ch, cw), generator=gen, device=device, dtype=torch.float64) * 32.0 - 16.0
        out.append(torch.clamp(torch.round(c + 512.0), 64, 960).to(torch.int32))
    return tuple(out)


def yuv420p10_frames(h: int, w: int, t: int, seed: int = 7, distortion: str = "dct", device="cpu"):
    """(reference, distorted) YUV 4:2:0 10-bit frames for pair t of a sequence."""
    src = yuv420p10_source(h, w, t, seed, device)
    rs = np.random.default_rng([seed, t, 1])
    gen = torch.Generator(device=device).manual_seed(seed * 7919 + t)
    if distortion == "dct":
        step = rs.uniform(4.0, 32.0)
        dist = (block_dct_quantise(src[0], step, 64, 940),
                block_dct_quantise(src[1], 2 * step, 64, 960),
                block_dct_quantise(src[2], 2 * step, 64, 960))
    elif distortion == "blur_noise":
        sigma = rs.uniform(0.5, 2.0)
        ns = rs.uniform(1.0, 6.0)
        dist = (gaussian_blur_noise(src[0], sigma, ns, 64, 940, gen),
                gaussian_blur_noise(src[1], sigma, ns, 64, 960, gen),
                gaussian_blur_noise(src[2], sigma, ns, 64, 960, gen))
    else:
        raise ValueError(distortion)
    return src, dist


def _upsample_chroma(c: torch.Tensor, h: int, w: int) -> torch.Tensor:
    """Bilinear 2x upsampling with MPEG-2 siting: chroma sample i sits on luma column 2i and
    halfway between luma rows 2j and 2j+1. Edge samples are clamped."""
    ch, cw = c.shape
    xs = torch.arange(w, dtype=torch.float64, device=c.device) / 2.0
    ys = (torch.arange(h, dtype=torch.float64, device=c.device) - 0.5) / 2.0
    x0 = torch.clamp(torch.floor(xs), 0, cw - 1).long()
    x1 = torch.clamp(x0 + 1, max=cw - 1)
    fx = torch.clamp(xs - x0.to(torch.float64), 0.0, 1.0)
    y0f = torch.floor(ys)
    fy = ys - y0f
    y0 = torch.clamp(y0f, 0, ch - 1).long()
    y1 = torch.clamp(y0f + 1, 0, ch - 1).long()
    cf = c.to(torch.float64)
    top = cf[y0][:, x0] * (1 - fx) + cf[y0][:, x1] * fx
    bot = cf[y1][:, x0] * (1 - fx) + cf[y1][:, x1] * fx
    return top * (1 - fy)[:, None] + bot * fy[:, None]


def yuv420p10_to_rgb(yuv, dtype=torch.float32) -> torch.Tensor:
    """BT.709 limited-range 10-bit 4:2:0 -> full-range gamma-encoded R'G'B' (3, h, w) in [0, 1]."""
    Y, U, V = yuv
    h, w = Y.shape
    y = (Y.to(torch.float64) - 64.0) / 876.0
    cb = (_upsample_chroma(U, h, w) - 512.0) / 896.0
    cr = (_upsample_chroma(V, h, w) - 512.0) / 896.0
    kr, kb = 0.2126, 0.0722
    kg = 1.0 - kr - kb
    r = y + 2.0 * (1.0 - kr) * cr
    b = y + 2.0 * (1.0 - kb) * cb
    g = y - (2.0 * (1.0 - kb) * kb / kg) * cb - (2.0 * (1.0 - kr) * kr / kg) * cr
    rgb = torch.stack([r, g, b]).clamp_(0.0, 1.0)
    return rgb.to(dtype)


# ------------------------------------------------------------------------------------------
# Y'CbCr of any depth / subsampling / matrix / range / chroma siting

_MATRICES = {1: (0.2126, 0.0722), 4: (0.30, 0.11), 5: (0.299, 0.114), 6: (0.299, 0.114), 7: (0.212, 0.087),
             9: (0.2627, 0.0593)}


def _range(bits: int, full: bool):
    sc = float(1 << (bits - 8))
    if full:
        mx = float((1 << bits) - 1)
        return 0.0, mx, float(1 << (bits - 1)), mx
    return 16.0 * sc, 219.0 * sc, 128.0 * sc, 224.0 * sc


def _siting(loc: int):
    """(horizontal, vertical) chroma siting in luma half-samples: 0 even positions, 1 halfway,
    2 odd positions (left, center, top-left, top, bottom-left, bottom)."""
    sx = 1 if loc in (1, 3, 5) else 0
    sy = 1 if loc <= 1 else (0 if loc <= 3 else 2)
    return sx, sy


def _upsample_axis(c: torch.Tensor, n: int, ss: int, s: int, axis: int) -> torch.Tensor:
    if not ss:
        return c
    m = c.shape[axis]
    p = torch.arange(n, dtype=torch.float64, device=c.device)
    pos = (2 * p - s) / 4.0  # chroma sample k sits at luma position 2k + s/2
    k0f = torch.floor(pos)
    f = pos - k0f
    k0 = torch.clamp(k0f, 0, m - 1).long()
    k1 = torch.clamp(k0f + 1, 0, m - 1).long()
    a, b = c.index_select(axis, k0), c.index_select(axis, k1)
    shape = [1, 1]
    shape[axis] = n
    f = f.view(shape)
    return a * (1 - f) + b * f


def _bt2020_to_bt709() -> np.ndarray:
    def npm(xy):
        P = np.array([[x / y for x, y in xy[:3]], [1.0, 1.0, 1.0], [(1 - x - y) / y for x, y in xy[:3]]])
        wx, wy = xy[3]
        W = np.array([wx / wy, 1.0, (1 - wx - wy) / wy])
        return P * np.linalg.solve(P, W)[None, :]
    d65 = (0.3127, 0.3290)
    a = npm([(0.640, 0.330), (0.300, 0.600), (0.150, 0.060), d65])
    b = npm([(0.708, 0.292), (0.170, 0.797), (0.131, 0.046), d65])
    return np.linalg.solve(a, b)


def _eotf(v: torch.Tensor, transfer: int) -> torch.Tensor:
    a = v.abs()
    if transfer == 13:
        l = torch.where(a <= 0.04045, a / 12.92, ((a + 0.055) / 1.055) ** 2.4)
    elif transfer in (4, 5):
        l = a ** (2.2 if transfer == 4 else 2.8)
    elif transfer == 8:
        l = a
    else:
        l = a ** 2.4
    return torch.sign(v) * l


def yuv_to_rgb(yuv, bits=10, ssw=1, ssh=1, matrix=1, full=False, loc=0, dtype=torch.float32, transfer=1,
               primaries=1) -> torch.Tensor:
    """Y'CbCr planes of the given format -> full-range R'G'B' (3, h, w) in [0, 1], in FP64: chroma
    upsampled bilinearly at its siting (edge samples clamped), the matrix (H.273 id; 2 = BT.709
    above 650 rows, BT.470BG below) and range applied, clamped. A transfer outside the BT.709
    family (H.273 13 sRGB, 4 / 5 gamma 2.2 / 2.8, 8 linear) or BT.2020 primaries (9): the samples
    go to linear light, to BT.709 primaries, are clamped there, and come back as the 2.4 power law
    the metrics linearise with."""
    Y, U, V = [p.to(torch.float64) for p in yuv]
    h, w = Y.shape
    if matrix == 2:
        matrix = 1 if h > 650 else 5
    kr, kb = _MATRICES[matrix]
    kg = 1.0 - kr - kb
    yo, yd, co, cd = _range(bits, full)
    sx, sy = _siting(loc)
    ups = lambda c: _upsample_axis(_upsample_axis(c, w, ssw, sx, 1), h, ssh, sy, 0)
    y = (Y - yo) / yd
    cb = (ups(U) - co) / cd
    cr = (ups(V) - co) / cd
    r = y + 2.0 * (1.0 - kr) * cr
    b = y + 2.0 * (1.0 - kb) * cb
    g = y - (2.0 * (1.0 - kb) * kb / kg) * cb - (2.0 * (1.0 - kr) * kr / kg) * cr
    rgb = torch.stack([r, g, b])
    if transfer in (1, 2, 6, 14, 15) and primaries in (1, 2):
        return rgb.clamp_(0.0, 1.0).to(dtype)
    lin = _eotf(rgb, transfer)
    if primaries == 9:
        m = torch.from_numpy(_bt2020_to_bt709()).to(lin)
        lin = torch.einsum("ij,jhw->ihw", m, lin)
    return lin.clamp_(0.0, 1.0).pow_(1.0 / 2.4).to(dtype)


def yuv_frames(h: int, w: int, t: int, bits=10, ssw=1, ssh=1, full=False, seed: int = 7, distortion="dct",
               device="cpu"):
    """(reference, distorted) Y'CbCr frames (int32 planes) of the given depth, subsampling and
    range: the grating model of yuv420p10_source at that depth, distorted by 8x8 block-DCT
    quantisation or by blur + noise, clipped to the range's codes."""
    rs = np.random.default_rng([seed, bits, ssw, ssh, int(full)])
    gen = torch.Generator(device=device).manual_seed(seed * 7919 + t)
    sc = float(1 << (bits - 8))
    top = (1 << bits) - 1
    ylo, yhi = (0, top) if full else (int(16 * sc), int(235 * sc))
    clo, chi = (0, top) if full else (int(16 * sc), int(240 * sc))
    ch, cw = ((h + 1) // 2 if ssh else h), ((w + 1) // 2 if ssw else w)
    yv = _gratings(h, w, rs, 8, 0.6 * sc, 0.05 * t, device) + 125.0 * sc
    yv += torch.rand((h, w), generator=gen, device=device, dtype=torch.float64) * 16 * sc - 8 * sc
    planes = [torch.clamp(torch.round(yv), ylo, yhi).to(torch.int32)]
    for _ in range(2):
        c = _gratings(ch, cw, rs, 8, 0.5 * sc, 0.05 * t, device) + 128.0 * sc
        c += torch.rand((ch, cw), generator=gen, device=device, dtype=torch.float64) * 8 * sc - 4 * sc
        planes.append(torch.clamp(torch.round(c), clo, chi).to(torch.int32))
    if distortion == "dct":
        step = rs.uniform(4.0, 32.0) * sc
        dist = [block_dct_quantise(planes[0], step, ylo, yhi)] + \
               [block_dct_quantise(p, 2 * step, clo, chi) for p in planes[1:]]
    else:
        sigma, ns = rs.uniform(0.5, 2.0), rs.uniform(1.0, 6.0) * sc
        dist = [gaussian_blur_noise(planes[0], sigma, ns, ylo, yhi, gen)] + \
               [gaussian_blur_noise(p, sigma, ns, clo, chi, gen) for p in planes[1:]]
    return tuple(planes), tuple(dist)


def rgb_float_pair(h: int, w: int, t: int, seed: int = 7, distortion: str = "dct", device="cpu"):
    """Float32 (3, h, w) R'G'B' reference/distorted planes for pair t of a YUV sequence."""
    ref, dist = yuv420p10_frames(h, w, t, seed, distortion, device)
    return yuv420p10_to_rgb(ref), yuv420p10_to_rgb(dist)


def write_y4m(path: str, frames, w: int, h: int, bits: int = 10, fps: str = "24:1", chroma: str = "420",
              siting: str = "") -> None:
    """Write frames [(Y, Cb, Cr) integer arrays] as YUV4MPEG2: chroma "420", "422" or "444";
    8-bit samples in bytes, deeper ones in little-endian 16-bit containers. The colorspace tag is
    C<chroma><siting> for 8 bits (siting "jpeg", "mpeg2", "paldv" or "" for 4:2:0) and
    C<chroma>p<bits> above."""
    import numpy as np

    tag = f"C{chroma}{siting}" if bits == 8 else f"C{chroma}p{bits}"
    if chroma == "420" and bits == 8 and not siting:
        tag = "C420jpeg"
    with open(path, "wb") as f:
        f.write(f"YUV4MPEG2 W{w} H{h} F{fps} Ip A1:1 {tag}\n".encode())
        for fr in frames:
            f.write(b"FRAME\n")
            for p in fr:
                a = np.asarray(p.cpu().numpy() if hasattr(p, "cpu") else p)
                f.write(a.astype("<u2" if bits > 8 else "u1").tobytes())
