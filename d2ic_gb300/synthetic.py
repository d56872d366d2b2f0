"""Seeded synthetic speckle images and deformation fields.

These stand in for the DIC-Challenge / PlateHole images that the reference's
benchmark and validation scripts read from TIFF files (no image decoder and
no dataset are available here).  A speckle pattern is a sum of Gaussian dots
(``H*W/12`` dots, centres uniform over the image, sigma ~ U[1.5, 3] px,
amplitude ~ U[0.5, 1]), scaled to grey levels [20, 230] with the reference
image's min/max, plus fresh N(0, noise^2) noise per image.  A deformed image
re-evaluates the same dot field at ``phi^{-1}(y)`` for each pixel centre ``y``,
so brightness constancy ``I2(phi(x)) = I1(x)`` holds exactly (up to noise).

Coordinates: pixel (i, j) has centre (x, y) = (j + 0.5, i + 0.5), as in the
reference (d2ic/pixel_assets.py:131).

Rendering runs in torch float64 on any device (CPU for tests, CUDA for large
benchmark frames); on CUDA the splat uses atomics, so two renders can differ
in the last bits, but a rendered image is a fixed input for every consumer.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

CUTOFF_SIGMAS = 4.5


@dataclass
class DotField:
    cx: np.ndarray
    cy: np.ndarray
    sigma: np.ndarray
    amp: np.ndarray


def make_dots(H: int, W: int, seed: int) -> DotField:
    rng = np.random.default_rng(seed)
    n = (H * W) // 12
    cx = rng.uniform(0.0, W, n)
    cy = rng.uniform(0.0, H, n)
    sigma = rng.uniform(1.5, 3.0, n)
    amp = rng.uniform(0.5, 1.0, n)
    return DotField(cx, cy, sigma, amp)


# ---------------------------------------------------------------------------
# deformation maps: forward phi(x) and inverse phi^{-1}(y), on (n,2) torch tensors
# ---------------------------------------------------------------------------

class Translation:
    def __init__(self, tx: float, ty: float):
        self.t = (float(tx), float(ty))

    def forward(self, xy):
        return xy + torch.tensor(self.t, dtype=xy.dtype, device=xy.device)

    def inverse(self, xy):
        return xy - torch.tensor(self.t, dtype=xy.dtype, device=xy.device)

    def displacement(self, xy):
        return torch.tensor(self.t, dtype=xy.dtype, device=xy.device).expand_as(xy).clone()

    max_stretch = 1.0


class Affine:
    """``phi(x) = x + A (x - x0) + t``."""

    def __init__(self, A, t, x0):
        self.A = np.asarray(A, dtype=np.float64).reshape(2, 2)
        self.t = np.asarray(t, dtype=np.float64)
        self.x0 = np.asarray(x0, dtype=np.float64)
        self.Minv = np.linalg.inv(np.eye(2) + self.A)
        self.max_stretch = float(np.linalg.norm(np.eye(2) + self.A, 2))

    def forward(self, xy):
        A = torch.tensor(self.A, dtype=xy.dtype, device=xy.device)
        x0 = torch.tensor(self.x0, dtype=xy.dtype, device=xy.device)
        t = torch.tensor(self.t, dtype=xy.dtype, device=xy.device)
        return xy + (xy - x0) @ A.T + t

    def inverse(self, xy):
        Mi = torch.tensor(self.Minv, dtype=xy.dtype, device=xy.device)
        x0 = torch.tensor(self.x0, dtype=xy.dtype, device=xy.device)
        t = torch.tensor(self.t, dtype=xy.dtype, device=xy.device)
        return x0 + (xy - x0 - t) @ Mi.T

    def displacement(self, xy):
        return self.forward(xy) - xy


class PlateHoleField:
    """``u(x,y) = t [0.01 (x - cx), -0.003 (y - cy)] + t * 2 sin(2 pi x / L) * e_y``.

    The x-component depends on x only and the y-component is affine in y, so
    the inverse is closed form.
    """

    def __init__(self, t: float, cx: float = 1024.0, cy: float = 1024.0, L: float = 2048.0):
        self.t, self.cx, self.cy, self.L = float(t), float(cx), float(cy), float(L)
        self.max_stretch = 1.0 + 0.01 * self.t + 2 * self.t * 2 * math.pi / self.L + 1e-3

    def displacement(self, xy):
        t = self.t
        ux = t * 0.01 * (xy[:, 0] - self.cx)
        uy = -t * 0.003 * (xy[:, 1] - self.cy) + t * 2.0 * torch.sin(2 * math.pi * xy[:, 0] / self.L)
        return torch.stack([ux, uy], dim=1)

    def forward(self, xy):
        return xy + self.displacement(xy)

    def inverse(self, xy):
        t = self.t
        x = (xy[:, 0] + t * 0.01 * self.cx) / (1.0 + 0.01 * t)
        y = (xy[:, 1] - t * 0.003 * self.cy - t * 2.0 * torch.sin(2 * math.pi * x / self.L)) / (1.0 - 0.003 * t)
        return torch.stack([x, y], dim=1)


# ---------------------------------------------------------------------------
# rendering
# ---------------------------------------------------------------------------

def render_dots(H: int, W: int, dots: DotField, warp=None, device="cpu", batch: int = 65536) -> torch.Tensor:
    """Sum of Gaussian dots sampled at ``phi^{-1}(pixel centre)`` (identity if ``warp`` is None).

    Each dot contributes to pixels whose back-mapped centre lies within
    ``CUTOFF_SIGMAS * sigma`` of the dot centre (cut-off applied in the
    reference frame, so the warped image is exactly the warped field).
    """
    dev = torch.device(device)
    img = torch.zeros(H * W, dtype=torch.float64, device=dev)
    cx = torch.as_tensor(dots.cx, dtype=torch.float64, device=dev)
    cy = torch.as_tensor(dots.cy, dtype=torch.float64, device=dev)
    sg = torch.as_tensor(dots.sigma, dtype=torch.float64, device=dev)
    am = torch.as_tensor(dots.amp, dtype=torch.float64, device=dev)
    stretch = 1.0 if warp is None else float(getattr(warp, "max_stretch", 1.05))
    if warp is not None:
        fc = warp.forward(torch.stack([cx, cy], dim=1))
        fx, fy = fc[:, 0], fc[:, 1]
    else:
        fx, fy = cx, cy
    R = int(math.ceil(CUTOFF_SIGMAS * float(dots.sigma.max()) * stretch)) + 1
    off = torch.arange(-R, R + 1, device=dev)
    oy, ox = torch.meshgrid(off, off, indexing="ij")
    ox = ox.reshape(-1)
    oy = oy.reshape(-1)
    n = cx.shape[0]
    for s in range(0, n, batch):
        e = min(n, s + batch)
        # pixel containing the (forward-mapped) dot centre
        j0 = torch.floor(fx[s:e]).long()
        i0 = torch.floor(fy[s:e]).long()
        jj = j0[:, None] + ox[None, :]
        ii = i0[:, None] + oy[None, :]
        inb = (jj >= 0) & (jj < W) & (ii >= 0) & (ii < H)
        px = jj.to(torch.float64) + 0.5
        py = ii.to(torch.float64) + 0.5
        if warp is not None:
            q = warp.inverse(torch.stack([px.reshape(-1), py.reshape(-1)], dim=1))
            qx = q[:, 0].reshape(px.shape)
            qy = q[:, 1].reshape(py.shape)
        else:
            qx, qy = px, py
        d2 = (qx - cx[s:e, None]) ** 2 + (qy - cy[s:e, None]) ** 2
        s2 = sg[s:e, None] ** 2
        keep = inb & (d2 <= (CUTOFF_SIGMAS ** 2) * s2)
        val = am[s:e, None] * torch.exp(-d2 / (2.0 * s2))
        flat = (ii * W + jj)[keep]
        img.index_add_(0, flat, val[keep])
    return img.reshape(H, W)


def speckle_sequence(H: int, W: int, warps, seed: int, noise_seeds, noise_sigma: float = 1.0,
                     device="cpu", dtype=np.float32):
    """Reference image plus one deformed image per warp, as numpy arrays.

    ``noise_seeds[0]`` seeds the reference image's noise, ``noise_seeds[k+1]``
    that of deformed frame k.  Grey levels are scaled to [20, 230] with the
    noise-free reference image's min/max, reused for every deformed frame.
    """
    dots = make_dots(H, W, seed)
    ref = render_dots(H, W, dots, None, device)
    lo, hi = float(ref.min()), float(ref.max())
    scale = 210.0 / max(hi - lo, 1e-12)

    def finish(img, nseed):
        g = 20.0 + (img - lo) * scale
        rng = np.random.default_rng(nseed)
        out = g.cpu().numpy() + rng.normal(0.0, noise_sigma, size=(H, W))
        return out.astype(dtype)

    ref_np = finish(ref, noise_seeds[0])
    frames = []
    for k, wp in enumerate(warps):
        frames.append(finish(render_dots(H, W, dots, wp, device), noise_seeds[k + 1]))
    return ref_np, frames


# ---------------------------------------------------------------------------
# device rendering (benchmark streams): the same dot field and cut-off, FP32 sums
# in a fixed order per pixel, affine maps only
# ---------------------------------------------------------------------------

def _inverse_affine6(warp) -> np.ndarray:
    """``x = phi^{-1}(y)`` as ``(m0, m1, m2, m3, m4, m5)``: x = m0 + m1 yx + m2 yy, y = m3 + m4 yx + m5 yy."""
    if warp is None:
        M, off = np.eye(2), np.zeros(2)
    elif isinstance(warp, Translation):
        M, off = np.eye(2), -np.asarray(warp.t, np.float64)
    elif isinstance(warp, Affine):
        M = warp.Minv
        off = warp.x0 - M @ (warp.x0 + warp.t)
    else:
        raise ValueError("device rendering supports Translation and Affine maps")
    return np.array([off[0], M[0, 0], M[0, 1], off[1], M[1, 0], M[1, 1]], np.float64)


class DeviceSpeckle:
    """A dot field bucketed on the host into cells of ``cell_px`` pixels and kept on the device;
    renders raw fields (``d2ic_render_speckle``) and finished grey-level frames."""

    def __init__(self, H: int, W: int, dots: DotField, device, cell_px: float = 16.0):
        from . import _lib
        self.H, self.W, self.device = H, W, torch.device(device)
        if cell_px < CUTOFF_SIGMAS * float(dots.sigma.max()):
            raise ValueError("cells must be at least as wide as the largest cut-off radius")
        gw, gh = int(math.ceil(W / cell_px)) + 1, int(math.ceil(H / cell_px)) + 1
        cx = np.minimum((dots.cx // cell_px).astype(np.int64), gw - 1)
        cy = np.minimum((dots.cy // cell_px).astype(np.int64), gh - 1)
        cell = cy * gw + cx
        order = np.argsort(cell, kind="stable")
        start = np.zeros(gw * gh + 1, np.int32)
        start[1:] = np.cumsum(np.bincount(cell, minlength=gw * gh))
        d4 = np.stack([dots.cx, dots.cy, dots.sigma, dots.amp], axis=1)[order].astype(np.float32)
        self.dots = torch.from_numpy(np.ascontiguousarray(d4)).to(self.device)
        self.start = torch.from_numpy(start).to(self.device)
        self.gw, self.gh, self.cell_px = gw, gh, float(cell_px)
        self._lib = _lib

    def raw(self, warp=None, out: torch.Tensor | None = None) -> torch.Tensor:
        import ctypes

        from ._lib import ptr
        out = torch.empty((self.H, self.W), dtype=torch.float32, device=self.device) if out is None else out
        m = np.ascontiguousarray(_inverse_affine6(warp), dtype=np.float64)     # host array: read by the host
        self._lib.call("d2ic_render_speckle", ptr(self.dots), ptr(self.start), self.cell_px, self.gw, self.gh,
                       CUTOFF_SIGMAS, m.ctypes.data_as(ctypes.c_void_p), self.H, self.W, ptr(out),
                       self._lib.stream_handle())
        return out

    def finish(self, raw: torch.Tensor, lo: float, scale: float, sigma: float, seed: int, u8: bool) -> torch.Tensor:
        from ._lib import ptr
        out = torch.empty(raw.shape, dtype=torch.uint8 if u8 else torch.float32, device=self.device)
        self._lib.call("d2ic_speckle_finish", ptr(raw), raw.numel(), float(lo), float(scale), float(sigma),
                       int(seed) & 0xFFFFFFFFFFFFFFFF, int(u8), ptr(out), self._lib.stream_handle())
        return out


def speckle_sequence_device(H: int, W: int, warps, seed: int, noise_seeds, noise_sigma: float = 0.5,
                            device="cuda", u8: bool = True):
    """Reference image and deformed frames rendered on the device (device tensors).

    Same dot field (seed ``seed``), cut-off and grey-level scaling as :func:`speckle_sequence`;
    the noise comes from the device generator seeded by ``noise_seeds`` and, with ``u8``, frames
    are rounded to 8-bit camera pixels."""
    sp = DeviceSpeckle(H, W, make_dots(H, W, seed), device)
    raw = sp.raw(None)
    lo, hi = (float(v) for v in torch.aminmax(raw))
    scale = 210.0 / max(hi - lo, 1e-12)
    ref = sp.finish(raw, lo, scale, noise_sigma, noise_seeds[0], u8)
    frames = [sp.finish(sp.raw(w, raw), lo, scale, noise_sigma, noise_seeds[k + 1], u8) for k, w in enumerate(warps)]
    return ref, frames


# ---------------------------------------------------------------------------
# benchmark masks
# ---------------------------------------------------------------------------

def rect_mask(H: int, W: int, h: int, w: int) -> np.ndarray:
    """Centred ``h x w`` rectangle."""
    m = np.zeros((H, W), dtype=bool)
    i0 = (H - h) // 2
    j0 = (W - w) // 2
    m[i0:i0 + h, j0:j0 + w] = True
    return m


def plate_hole_mask(H: int = 2048, W: int = 2048, side: int = 1800, radius: float = 300.0) -> np.ndarray:
    """Centred square minus a centred disk (pixel centres tested)."""
    m = rect_mask(H, W, side, side)
    r2 = (np.arange(W)[None, :] + 0.5 - W / 2) ** 2 + (np.arange(H)[:, None] + 0.5 - H / 2) ** 2
    return m & (r2 >= radius * radius)


def ellipse_mask(H: int, W: int, rng: np.random.Generator, cover_lo=0.4, cover_hi=0.9) -> np.ndarray:
    """Axis-aligned centred ellipse covering a uniform fraction of the image."""
    cover = rng.uniform(cover_lo, cover_hi)
    aspect = rng.uniform(0.75, 1.0)
    # area = pi a b = cover H W with b/a = aspect (clipped to the image)
    a = math.sqrt(cover * H * W / (math.pi * aspect))
    b = aspect * a
    a = min(a, W / 2 - 4)
    b = min(b, H / 2 - 4)
    tx = ((np.arange(W)[None, :] + 0.5 - W / 2) / a) ** 2          # the same terms per pixel, broadcast
    ty = ((np.arange(H)[:, None] + 0.5 - H / 2) / b) ** 2
    return tx + ty <= 1.0
