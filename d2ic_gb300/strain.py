"""Nodal Green-Lagrange strain on the GPU (reference: d2ic/strain.py:11-148)."""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import ptr


def _dev(x, dtype, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    npdt = np.float32 if dtype == torch.float32 else np.int32
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=npdt))).to(device)


def strain_device(u, nodes, nbr_index, nbr_degree, gauge_length=0.0, eps=1e-8, device=None, want_F=False):
    """Voigt strain ``[E11, E22, E12]`` (and F if requested) as CUDA tensors."""
    device = torch.device(device if device is not None else (u.device if isinstance(u, torch.Tensor) else "cuda"))
    ud = _dev(u, torch.float32, device).reshape(-1, 2)
    Xd = _dev(nodes, torch.float32, device).reshape(-1, 2)
    idx = _dev(nbr_index, torch.int32, device)
    n = ud.shape[0]
    idx = idx.reshape(n, -1)
    deg = _dev(nbr_degree, torch.int32, device).reshape(-1)
    voigt = torch.empty((n, 3), dtype=torch.float32, device=device)
    F = torch.empty((n, 2, 2), dtype=torch.float32, device=device) if want_F else None
    _lib.call("d2ic_strain_gl", ptr(ud), ptr(Xd), ptr(idx), ptr(deg), n, idx.shape[1], float(gauge_length),
              float(eps), ptr(voigt), ptr(F), _lib.stream_handle())
    return voigt, F


def compute_green_lagrange_strain_nodes_lsq(displacement, nodes_coord, node_neighbor_index, node_neighbor_degree,
                                            gauge_length: float = 0.0, eps: float = 1e-8):
    """``(F_all, E_all)`` each (Nn, 2, 2), weighted-LSQ deformation gradient and Green-Lagrange strain."""
    voigt, F = strain_device(displacement, nodes_coord, node_neighbor_index, node_neighbor_degree, gauge_length,
                             eps, want_F=True)
    v = voigt.cpu().numpy()
    E = np.empty((v.shape[0], 2, 2), dtype=np.float32)
    E[:, 0, 0] = v[:, 0]
    E[:, 1, 1] = v[:, 1]
    E[:, 0, 1] = v[:, 2]
    E[:, 1, 0] = v[:, 2]
    return F.cpu().numpy(), E


def green_lagrange_to_voigt(E_all):
    """``[E11, E22, E12]`` of the symmetric part of (N, 2, 2) tensors."""
    E = np.asarray(E_all)
    s = 0.5 * (E + np.swapaxes(E, 1, 2))
    return np.stack([s[:, 0, 0], s[:, 1, 1], s[:, 0, 1]], axis=1)


def small_strain_nodes_lsq(displacement, nodes_coord, node_neighbor_index, node_neighbor_degree,
                           gauge_length: float = 0.0, eps: float = 1e-8):
    """Green-Lagrange strain in Voigt form (equal to small strain for small gradients)."""
    voigt, _ = strain_device(displacement, nodes_coord, node_neighbor_index, node_neighbor_degree, gauge_length, eps)
    return voigt.cpu().numpy()
