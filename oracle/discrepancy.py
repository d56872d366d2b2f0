"""Oracle (test infrastructure only): the reference-domain discrepancy map.

Restates d2ic/discrepancy.py:12-48 (``bilinear_sample_numpy``) and :86-127
(``compute_discrepancy_map_ref``) in FP64 numpy: pixel displacement from the
pixel shape functions, bilinear samples with the reference's validity rule
(base index inside [0, H-2] x [0, W-2]), residuals scattered to the ROI pixels'
flat indices (mean over duplicates), NaN where no valid sample landed.
"""
from __future__ import annotations

import numpy as np


def bilinear_sample(image: np.ndarray, coords: np.ndarray) -> np.ndarray:
    image = np.asarray(image, dtype=np.float64)
    x = np.asarray(coords, dtype=np.float64)[:, 0] - 0.5
    y = np.asarray(coords, dtype=np.float64)[:, 1] - 0.5
    j0 = np.floor(x).astype(np.int64)
    i0 = np.floor(y).astype(np.int64)
    fx, fy = x - j0, y - i0
    H, W = image.shape
    valid = (i0 >= 0) & (i0 < H - 1) & (j0 >= 0) & (j0 < W - 1)
    out = np.full(x.shape[0], np.nan)
    i, j, a, b = i0[valid], j0[valid], fx[valid], fy[valid]
    out[valid] = (image[i, j] * (1 - a) * (1 - b) + image[i, j + 1] * a * (1 - b)
                  + image[i + 1, j] * (1 - a) * b + image[i + 1, j + 1] * a * b)
    return out


def discrepancy_map_ref(ref_image, def_image, u_nodal, pixel_coords_ref, pixel_nodes, pixel_shapeN, roi_flat,
                        image_shape):
    H, W = image_shape
    u = np.asarray(u_nodal, dtype=np.float64)
    disp = np.sum(np.asarray(pixel_shapeN, np.float64)[..., None] * u[np.asarray(pixel_nodes)], axis=1)
    pc = np.asarray(pixel_coords_ref, dtype=np.float64)
    r = bilinear_sample(def_image, pc + disp) - bilinear_sample(ref_image, pc)
    valid = np.isfinite(r)
    rms = float(np.sqrt(np.sum(np.where(valid, r, 0.0) ** 2) / max(int(valid.sum()), 1)))
    acc = np.bincount(roi_flat, weights=np.where(valid, r, 0.0), minlength=H * W)
    cnt = np.bincount(roi_flat, weights=valid.astype(np.float64), minlength=H * W)
    out = np.where(cnt > 0, acc / np.maximum(cnt, 1.0), np.nan)
    return out.reshape(H, W), rms
