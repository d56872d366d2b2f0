"""Benchmark workloads (seeded synthetic stand-ins for the reference's image sets).

* ``translation_512``: 512^2 speckle, uniform translation (0.35, -0.62) px,
  central 448^2 mask, 16 px elements, MeshDICConfig(200, 1e-3, 0.1).
* ``plate_hole_2048``: 2048^2 speckle, 1800^2 square minus an r = 300 disk,
  16 px elements, 20 frames of ``u = t [0.01 (x-1024), -0.003 (y-1024)] +
  t 2 sin(2 pi x / 2048) e_y`` with ``t = k/19``; frame 0 initialised by
  ZNCC (win 17 -- the reference rejects even windows --, search 8) + IDW,
  later frames warm-started from the previous solution; tol 1e-3, reg 0.1.

Seeds: reference image ``seed``; frame k noise ``100 + k`` (plate hole) /
``seed + 1`` (translation).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .dataclasses import InitMotionConfig, MeshDICConfig
from .mask2mesh import mask_to_mesh_assets
from .pixel_assets import build_pixel_assets
from .synthetic import PlateHoleField, Translation, plate_hole_mask, rect_mask, speckle_sequence


@dataclass
class Workload:
    name: str
    ref: np.ndarray
    frames: list
    mask: np.ndarray
    mesh: object
    assets: object
    config: MeshDICConfig
    init: InitMotionConfig | None
    fields: list = field(default_factory=list)    # ground-truth warps per frame

    @property
    def n_pix(self) -> int:
        return self.assets.pixel_data.n_pixels

    @property
    def n_nodes(self) -> int:
        return int(np.asarray(self.mesh.nodes_xy).shape[0])


def _build_assets(items, elems, workers: int | None = None):
    """Mesh + pixel assets of (mask, reference image) pairs on host threads (numpy releases the GIL)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    from dataclasses import replace

    def one(arg):
        (mask, ref), elem = arg
        mesh, assets = mask_to_mesh_assets(mask, elem)
        return mesh, replace(assets, pixel_data=build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))

    n = workers or min(16, os.cpu_count() or 1)
    with ThreadPoolExecutor(max_workers=n) as ex:
        return list(ex.map(one, zip(items, elems)))


def translation_512(seed: int = 0, device="cpu") -> Workload:
    H = W = 512
    warp = Translation(0.35, -0.62)
    ref, frames = speckle_sequence(H, W, [warp], seed=seed, noise_seeds=[seed, seed + 1], device=device)
    mask = rect_mask(H, W, 448, 448)
    mesh, assets = mask_to_mesh_assets(mask, 16)
    from dataclasses import replace
    assets = replace(assets, pixel_data=build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    return Workload("translation_512", ref, frames, mask, mesh, assets,
                    MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1), None, [warp])


def mixed_stream(n_seq: int = 16, frames_per_seq: int = 4, seed: int = 4, device="cpu",
                 sides=(512, 1024, 2048), elements=(8, 16, 32)):
    """Sequences of uneven size for the served form (seed ``seed``; sequence s uses ``4000 + s``).

    Per sequence: side and element size drawn uniformly, ellipse mask covering
    40-90%, a random affine map (strains +-2%, rotation +-1 deg, translation
    +-3 px) reached progressively (frame k at fraction (k+1)/frames_per_seq),
    N(0, 0.5^2) grey noise per image; frame 0 is initialised by ZNCC + IDW.
    """
    import math
    from dataclasses import replace

    from .synthetic import Affine, ellipse_mask
    rng = np.random.default_rng(seed)
    specs = []
    for s in range(n_seq):
        H = int(rng.choice(sides))
        elem = int(rng.choice(elements))
        r = np.random.default_rng(4000 + s)
        exx, eyy, exy = r.uniform(-0.02, 0.02, 3)
        th = math.radians(r.uniform(-1.0, 1.0))
        t = r.uniform(-3.0, 3.0, 2)
        A = np.array([[exx, exy], [exy, eyy]]) + np.array([[math.cos(th) - 1, -math.sin(th)],
                                                          [math.sin(th), math.cos(th) - 1]])
        warps = [Affine(A * (k + 1) / frames_per_seq, t * (k + 1) / frames_per_seq, [H / 2, H / 2])
                 for k in range(frames_per_seq)]
        ref, frames = speckle_sequence(H, H, warps, seed=4000 + s, noise_seeds=[40000 + 100 * s + k for k in
                                                                                 range(frames_per_seq + 1)],
                                       noise_sigma=0.5, device=device)
        specs.append((s, H, elem, ref, frames, ellipse_mask(H, H, r), warps))
    built = _build_assets([(sp[5], sp[3]) for sp in specs], [sp[2] for sp in specs])
    return [Workload(f"seq{s}_{H}px_e{elem}", ref, frames, mask, mesh, assets,
                     MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1),
                     InitMotionConfig(win=17, search=8, score_min=0.2), warps)
            for (s, H, elem, ref, frames, mask, warps), (mesh, assets) in zip(specs, built)]


@dataclass
class StreamSequence:
    """One sequence of the serving stream: reference image (uint8, host), mesh and assets, and
    its frames (uint8, pinned host tensors) in the order they arrive."""
    seq_id: int
    side: int
    element_px: int
    ref: np.ndarray
    mesh: object
    assets: object
    frames: list
    config: MeshDICConfig
    init: InitMotionConfig
    warps: list


@dataclass
class ServingStream:
    """Arrival order of a serving stream: ``order[i] = (sequence, frame index)`` of arrival i."""
    sequences: list
    order: list
    seed: int

    def offsets(self, rate: float, n: int | None = None, seed: int | None = None) -> np.ndarray:
        """Poisson arrival times (seconds from the start) of the first ``n`` arrivals at ``rate``."""
        n = len(self.order) if n is None else n
        rng = np.random.default_rng((self.seed if seed is None else seed) * 100003 + int(round(rate)))
        return np.cumsum(rng.exponential(1.0 / rate, n))

    @property
    def host_bytes(self) -> int:
        return sum(int(f.numel()) for s in self.sequences for f in s.frames)


def serving_stream(n_arrivals: int = 4096, n_seq: int = 128, seed: int = 4, device="cuda",
                   sides=(512, 1024, 2048, 4096), elements=(8, 16, 32), noise_sigma: float = 0.5,
                   pin: bool = True, device_assets: bool = True) -> ServingStream:
    """The serving stream: ``n_arrivals`` frames from ``n_seq`` concurrent sequences.

    Seed ``seed`` draws each sequence's image side and element size (uniform over ``sides`` and
    ``elements``), then the sequence of every arrival (uniform over sequences; a sequence's
    frames arrive in order).  Sequence s uses seed ``4000 + s`` for its speckle, its ellipse mask
    (40-90% of the image) and its random affine map (strains +-2%, rotation +-1 deg, translation
    +-3 px about the centre), reached linearly over its frames: frame k of F shows the map at
    fraction (k + 1) / F.  Frames are 8-bit camera images with N(0, noise_sigma^2) grey noise,
    rendered on the device and kept in pinned host memory; frame 0 of a sequence is initialised
    by ZNCC + IDW, later frames warm-start from the previous solution.  ``device_assets``: pixel
    assets as device-layout recipes (build_pixel_assets_device) instead of host arrays."""
    import math
    from dataclasses import replace

    import torch

    from .synthetic import Affine, ellipse_mask, speckle_sequence_device
    rng = np.random.default_rng(seed)
    side = [int(rng.choice(sides)) for _ in range(n_seq)]
    elem = [int(rng.choice(elements)) for _ in range(n_seq)]
    seq_of = rng.integers(0, n_seq, n_arrivals)
    counts = np.bincount(seq_of, minlength=n_seq)
    order, seen = [], np.zeros(n_seq, np.int64)
    for s in seq_of:
        order.append((int(s), int(seen[s])))
        seen[s] += 1
    specs = []
    for s in range(n_seq):
        H, F = side[s], max(int(counts[s]), 1)
        r = np.random.default_rng(4000 + s)
        exx, eyy, exy = r.uniform(-0.02, 0.02, 3)
        th = math.radians(r.uniform(-1.0, 1.0))
        t = r.uniform(-3.0, 3.0, 2)
        A = np.array([[exx, exy], [exy, eyy]]) + np.array([[math.cos(th) - 1, -math.sin(th)],
                                                          [math.sin(th), math.cos(th) - 1]])
        warps = [Affine(A * (k + 1) / F, t * (k + 1) / F, [H / 2, H / 2]) for k in range(int(counts[s]))]
        ref_d, frames_d = speckle_sequence_device(H, H, warps, seed=4000 + s,
                                                  noise_seeds=[4_000_000 + 10_000 * s + k for k in range(len(warps) + 1)],
                                                  noise_sigma=noise_sigma, device=device, u8=True)
        frames = []
        for f in frames_d:
            h = torch.empty(f.shape, dtype=torch.uint8, pin_memory=pin)
            h.copy_(f)
            frames.append(h)
        ref = ref_d.cpu().numpy()
        specs.append((s, H, elem[s], ref, frames, ellipse_mask(H, H, r), warps))
    if device_assets:
        from .pixel_assets import build_pixel_assets_device
        built = []
        for sp in specs:
            mesh, assets = mask_to_mesh_assets(sp[5], sp[2])
            built.append((mesh, replace(assets, pixel_data=build_pixel_assets_device(mesh, sp[3], 1.0,
                                                                                      assets.roi_mask))))
    else:
        built = _build_assets([(sp[5], sp[3].astype(np.float32)) for sp in specs], [sp[2] for sp in specs])
    seqs = [StreamSequence(s, H, e, ref, mesh, assets, frames,
                           MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1),
                           InitMotionConfig(win=17, search=8, score_min=0.2), warps)
            for (s, H, e, ref, frames, mask, warps), (mesh, assets) in zip(specs, built)]
    return ServingStream(seqs, order, seed)


def plate_hole_2048(n_frames: int = 20, seed: int = 1, device="cpu", H: int = 2048) -> Workload:
    W = H
    s = H / 2048.0
    warps = [PlateHoleField(k / 19.0, cx=1024 * s, cy=1024 * s, L=2048 * s) for k in range(n_frames)]
    ref, frames = speckle_sequence(H, W, warps, seed=seed, noise_seeds=[seed] + [100 + k for k in range(n_frames)],
                                   device=device)
    mask = plate_hole_mask(H, W, int(round(1800 * s)), 300.0 * s)
    mesh, assets = mask_to_mesh_assets(mask, 16)
    from dataclasses import replace
    assets = replace(assets, pixel_data=build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    return Workload("plate_hole_2048" if H == 2048 else f"plate_hole_{H}", ref, frames, mask, mesh, assets,
                    MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1),
                    InitMotionConfig(win=17, search=8, score_min=0.2), warps)


def uneven_batch(n_frames: int = 64, seed: int = 2, device="cpu", sides=(512, 1024, 2048, 3072, 4096),
                 elements=(8, 12, 16, 24, 32), device_assets: bool = False):
    """Independent frames of uneven size for one batched launch (frame i uses seed ``2000 + i``).

    Per frame: side and element size drawn uniformly, ellipse mask covering
    40-90%, a random affine map (strains +-2%, rotation +-1 deg, translation
    +-3 px) about the image centre, N(0, 0.5^2) grey noise on both images.
    ``device_assets``: images rendered on the device (float32, the device noise generator) and
    pixel assets as device-layout recipes (build_pixel_assets_device) instead of host arrays.
    """
    import math
    from dataclasses import replace

    from .synthetic import Affine, ellipse_mask, speckle_sequence_device
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_frames):
        H = int(rng.choice(sides))
        elem = int(rng.choice(elements))
        r = np.random.default_rng(2000 + i)
        exx, eyy, exy = r.uniform(-0.02, 0.02, 3)
        th = math.radians(r.uniform(-1.0, 1.0))
        t = r.uniform(-3.0, 3.0, 2)
        A = np.array([[exx, exy], [exy, eyy]]) + np.array([[math.cos(th) - 1, -math.sin(th)],
                                                          [math.sin(th), math.cos(th) - 1]])
        warp = Affine(A, t, [H / 2, H / 2])
        if device_assets:
            ref_d, frames = speckle_sequence_device(H, H, [warp], seed=2000 + i,
                                                    noise_seeds=[20000 + 2 * i, 20001 + 2 * i],
                                                    noise_sigma=0.5, device=device, u8=False)
            ref = ref_d.cpu().numpy()
        else:
            ref, frames = speckle_sequence(H, H, [warp], seed=2000 + i, noise_seeds=[20000 + 2 * i, 20001 + 2 * i],
                                           noise_sigma=0.5, device=device)
        specs.append((i, H, elem, ref, frames, ellipse_mask(H, H, r), warp))
    if device_assets:
        from .pixel_assets import build_pixel_assets_device
        built = []
        for sp in specs:
            mesh, assets = mask_to_mesh_assets(sp[5], sp[2])
            built.append((mesh, replace(assets, pixel_data=build_pixel_assets_device(mesh, sp[3], 1.0,
                                                                                      assets.roi_mask))))
    else:
        built = _build_assets([(sp[5], sp[3]) for sp in specs], [sp[2] for sp in specs])
    return [Workload(f"frame{i}_{H}px_e{elem}", ref, frames, mask, mesh, assets,
                     MeshDICConfig(max_iters=200, tol=1e-3, reg_strength=0.1), None, [warp])
            for (i, H, elem, ref, frames, mask, warp), (mesh, assets) in zip(specs, built)]


def uniaxial_1024(seed: int = 3, device="cpu") -> Workload:
    """1024^2 speckle, centred 900^2 mask, 12 px elements, uniform 0.5% uniaxial strain (x)."""
    from dataclasses import replace

    from .synthetic import Affine
    H = W = 1024
    warp = Affine(np.array([[0.005, 0.0], [0.0, 0.0]]), np.zeros(2), [H / 2, W / 2])
    ref, frames = speckle_sequence(H, W, [warp], seed=seed, noise_seeds=[seed, seed + 1], device=device)
    mask = rect_mask(H, W, 900, 900)
    mesh, assets = mask_to_mesh_assets(mask, 12)
    assets = replace(assets, pixel_data=build_pixel_assets(mesh, ref, 1.0, assets.roi_mask))
    return Workload("uniaxial_1024", ref, frames, mask, mesh, assets,
                    MeshDICConfig(max_iters=400, tol=1e-5, reg_strength=0.1), None, [warp])
