"""Implicit-function adjoint of the converged global-CG solve.

The reference propagates image noise with ``jax.jvp`` through 25 unrolled
iterations of its nonlinear CG (doc/11_Advanced_Use_Uncertainty_Propagation.ipynb,
cells 14, 22, 24, 30).  Here the derivative of the converged solution u*(I2)
(grad_u J(u*, I2) = 0) is taken by the implicit function theorem:

    du* = -H^-1 (d grad_u J / dI2) dI,         dL/dI2 = -(d grad_u J / dI2)^T H^-1 dL/du*,

with H the exact Hessian of J at u* (pixel term with the residual times the
image Hessian, plus springs).  All heavy pieces are CUDA kernels of the
library: one pixel pass assembles per-chunk element blocks of H, H V for many
right-hand sides runs on those blocks (chunk -> slot -> node, no atomics), the
mixed term is a pixel pass over an image direction's B-spline coefficients and
its adjoint is the backward of the bicubic sampling (scatter + transposed
prefilter).  The right-hand sides of all noise realisations are solved
together by a block-Jacobi preconditioned CG (FP64 vectors, FP32 matvec).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import ptr
from .engine import PAD, FrameLayout, FrameSlot, descriptors_to_device, prepare_coefficients


def _pair(a, b):
    a, b = min(a, b), max(a, b)
    return a * 4 - (a * (a - 1)) // 2 + (b - a)


class ImplicitAdjoint:
    """Linearisation of one converged frame: JVP and VJP with respect to the deformed image."""

    def __init__(self, slot: FrameSlot, u_star, alpha_reg: float, exact: bool = True, stream=None):
        L: FrameLayout = slot.layout
        if L.kind != _lib.INTERP_CUBIC:
            raise ValueError("the adjoint is implemented for cubic interpolation")
        self.slot, self.L = slot, L
        self.dev = L.device
        self.alpha = float(alpha_reg)
        self.inv_np = 1.0 / max(L.n_pix, 1)
        self.u = torch.as_tensor(u_star, dtype=torch.float32, device=self.dev).reshape(-1, 2).contiguous()
        self.desc = descriptors_to_device([slot.desc], self.dev)
        self.hess = torch.empty(max(L.n_chunks, 1) * 32, dtype=torch.float32, device=self.dev)
        _lib.call("d2ic_hessian_chunks", ptr(self.desc), L.n_chunks, ptr(self.u), int(exact), ptr(self.hess),
                  _lib.stream_handle(stream))
        self._precond()
        self._slots_cap = 0
        self._slots = None

    # -- preconditioner: inverse 2x2 diagonal blocks, inactive dofs masked -------------------------------
    def _precond(self):
        L = self.L
        h = self.hess.cpu().numpy().reshape(-1, 32)[: L.n_chunks]
        cn = L.chunk_nodes.cpu().numpy().reshape(-1, 4)
        D = np.zeros((L.n_nodes, 3))
        for a in range(4):
            k = 3 * _pair(a, a)
            np.add.at(D, cn[:, a], h[:, k:k + 3] * self.inv_np)
        nbi = L.nbr_index.cpu().numpy().reshape(L.max_deg, L.n_nodes) if L.max_deg else np.zeros((0, L.n_nodes), int)
        nbw = L.nbr_weight.cpu().numpy().reshape(L.max_deg, L.n_nodes) if L.max_deg else np.zeros((0, L.n_nodes))
        spring = np.where(nbi >= 0, nbw, 0.0).sum(axis=0)
        D[:, 0] += self.alpha * spring
        D[:, 2] += self.alpha * spring
        det = D[:, 0] * D[:, 2] - D[:, 1] ** 2
        active = (np.abs(D).sum(axis=1) > 0) & (det > 0)
        inv = np.zeros((L.n_nodes, 2, 2))
        inv[active, 0, 0] = D[active, 2] / det[active]
        inv[active, 1, 1] = D[active, 0] / det[active]
        inv[active, 0, 1] = inv[active, 1, 0] = -D[active, 1] / det[active]
        self.Minv = torch.as_tensor(inv, dtype=torch.float64, device=self.dev).contiguous()
        self.active = torch.as_tensor(active, device=self.dev)
        self._active_u8 = self.active.to(torch.uint8).contiguous()
        self._pcg_work = None

    def operator(self) -> torch.Tensor:
        """The Hessian assembled into its node operator (d2ic_hessian_assemble), built once."""
        if getattr(self, "_op", None) is None:
            L = self.L
            nb = int(_lib.load().d2ic_hessian_op_bytes(L.n_nodes, L.node_chunk_k))
            self._op = torch.empty(nb, dtype=torch.uint8, device=self.dev)
            _lib.call("d2ic_hessian_assemble", ptr(self.desc), L.n_chunks, L.n_nodes, L.node_chunk_k, ptr(self.hess),
                      self.inv_np, self.alpha, ptr(self._op), nb, _lib.stream_handle())
        return self._op

    def apply(self, Vf: torch.Tensor, Y: torch.Tensor):
        """Y = H Vf for float32 (Nn, 2, K) tensors with the assembled operator."""
        L = self.L
        _lib.call("d2ic_hessian_apply", ptr(self.operator()), L.n_nodes, L.node_chunk_k, ptr(Vf), int(Vf.shape[2]),
                  ptr(Y), _lib.stream_handle())

    def matvec(self, V: torch.Tensor) -> torch.Tensor:
        """H V for V of shape (Nn, 2, K) (float64 in, float64 out; the kernels run in FP32)."""
        Vf = V.to(torch.float32).contiguous()
        Y = torch.empty_like(Vf)
        self.apply(Vf, Y)
        return Y.to(torch.float64)

    def matvec_chunks(self, V: torch.Tensor) -> torch.Tensor:
        """H V through the chunk blocks and node slots (d2ic_hessian_matvec, no assembly)."""
        L = self.L
        K = V.shape[2]
        Vf = V.to(torch.float32).contiguous()
        need = L.node_chunk_k * L.n_nodes * 2 * K
        if need > self._slots_cap:
            self._slots = torch.empty(need, dtype=torch.float32, device=self.dev)
            self._slots_cap = need
        self._slots[:need].zero_()            # slots that no chunk owns must read as 0 (layout depends on K)
        Y = torch.empty_like(Vf)
        _lib.call("d2ic_hessian_matvec", ptr(self.desc), L.n_chunks, L.n_nodes, ptr(self.hess), ptr(Vf), K,
                  self.inv_np, self.alpha, ptr(self._slots), ptr(Y), _lib.stream_handle())
        return Y.to(torch.float64)

    def solve(self, B: torch.Tensor, rtol: float = 1e-7, max_iter: int = 2000):
        """X = H^-1 B column by column: block-Jacobi PCG, all columns in lock step, run by
        ``d2ic_pcg_solve`` (FP64 vectors, FP32 Hessian matvec, deterministic reductions)."""
        import ctypes
        L = self.L
        B = B.to(device=self.dev, dtype=torch.float64).contiguous()
        K = int(B.shape[2])
        nb = _lib.load().d2ic_pcg_work_bytes(L.n_nodes, K, L.node_chunk_k)
        if self._pcg_work is None or self._pcg_work.numel() < nb:
            self._pcg_work = torch.empty(nb, dtype=torch.uint8, device=self.dev)
        X = torch.empty_like(B)
        it = ctypes.c_int(0)
        _lib.call("d2ic_pcg_solve", ptr(self.desc), L.n_chunks, L.n_nodes, L.node_chunk_k, ptr(self.hess),
                  self.inv_np, self.alpha, ptr(self.Minv), ptr(self._active_u8), ptr(B), ptr(X), K, float(rtol),
                  int(max_iter), ptr(self._pcg_work), self._pcg_work.numel(), ctypes.addressof(it),
                  _lib.stream_handle())
        self.last_iters = int(it.value)
        return X

    # -- the mixed term and its adjoint ---------------------------------------------------------------
    def _coeff(self, img: torch.Tensor) -> torch.Tensor:
        return prepare_coefficients(img.to(torch.float32).contiguous(), _lib.INTERP_CUBIC)

    MIXED_BATCH = 32   # images per launch of the batched prefilter and mixed term

    def mixed(self, dI: torch.Tensor) -> torch.Tensor:
        """(d grad_u J / dI2) dI_k for images dI (K, H, W) -> (Nn, 2, K): the images' B-spline
        coefficients and mixed terms in launches of up to MIXED_BATCH images (the same kernels and
        arithmetic as one image at a time)."""
        L = self.L
        K = dI.shape[0]
        H, W = L.H, L.W
        out = torch.empty((L.n_nodes, 2, K), dtype=torch.float32, device=self.dev)
        B = min(self.MIXED_BATCH, K)
        slots = torch.zeros(B * L.node_chunk_k * L.n_nodes * 2, dtype=torch.float32, device=self.dev)
        tmp = torch.empty((B, H, L.cpitch), dtype=torch.float32, device=self.dev)
        coeff = torch.empty((B, H + 2 * PAD, L.cpitch), dtype=torch.float32, device=self.dev)
        s = _lib.stream_handle()
        for k0 in range(0, K, B):
            nb = min(B, K - k0)
            imgs = dI[k0:k0 + nb].to(device=self.dev, dtype=torch.float32).contiguous()
            _lib.call("d2ic_bspline_prefilter_batch", ptr(imgs), nb, H, W, PAD, L.cpitch, ptr(tmp), ptr(coeff), s)
            _lib.call("d2ic_mixed_term_batch", ptr(self.desc), L.n_chunks, L.n_nodes, L.node_chunk_k, ptr(self.u),
                      ptr(coeff), nb, (H + 2 * PAD) * L.cpitch, self.inv_np, ptr(slots), ptr(out), K, k0, s)
        return out.to(torch.float64)

    def mixed_T(self, lam: torch.Tensor) -> torch.Tensor:
        """Adjoint: (Nn, 2, K) -> image-space (K, H, W)."""
        L = self.L
        K = lam.shape[2]
        out = torch.empty((K, L.H, L.W), dtype=torch.float32, device=self.dev)
        gco = torch.empty((L.H + 2 * PAD, L.cpitch), dtype=torch.float32, device=self.dev)
        tmp = torch.empty((L.H, L.cpitch), dtype=torch.float32, device=self.dev)
        for k in range(K):
            lk = lam[:, :, k].to(torch.float32).contiguous()
            gco.zero_()
            _lib.call("d2ic_mixed_term_T", ptr(self.desc), L.n_chunks, ptr(self.u), ptr(lk), self.inv_np, ptr(gco),
                      _lib.stream_handle())
            _lib.call("d2ic_bspline_prefilter_T", ptr(gco), L.H, L.W, PAD, L.cpitch, ptr(tmp), ptr(out[k]),
                      _lib.stream_handle())
        return out

    def jvp(self, dI: torch.Tensor, **kw) -> torch.Tensor:
        """du*/dI2 . dI for images (K, H, W) -> (K, Nn, 2)."""
        X = self.solve(self.mixed(dI), **kw)
        return (-X).permute(2, 0, 1).contiguous()

    def vjp(self, gu: torch.Tensor, **kw) -> torch.Tensor:
        """(du*/dI2)^T gu for gu (K, Nn, 2) -> (K, H, W)."""
        lam = self.solve(gu.to(torch.float64).permute(1, 2, 0).contiguous(), **kw)
        return -self.mixed_T(lam)


def newton_polish(solver, state, def_image, u, alpha_reg: float, steps: int = 3, exact: bool = True):
    """Refine a CG solution with exact Newton steps u <- u - H^-1 grad J (on the GPU)."""
    slot = solver._ensure(state)
    slot.load_image(def_image)
    u = torch.as_tensor(u, dtype=torch.float32, device=slot.layout.device).reshape(-1, 2).contiguous()
    for _ in range(steps):
        _, g = solver._engine.eval_objective(solver._desc_dev, u, solver._kind)
        adj = ImplicitAdjoint(slot, u, alpha_reg, exact)
        step = adj.solve(g.to(torch.float64).reshape(-1, 2, 1))[:, :, 0]
        u = (u.to(torch.float64) - step).to(torch.float32).contiguous()
    return u


def strain_jvp(u, du, nodes, nbr_index, nbr_degree, gauge_length: float = 0.0, eps: float = 1e-8):
    """Linearised Green-Lagrange Voigt strain: d voigt for displacement directions du (K, Nn, 2).

    Same weighted least squares as d2ic/strain.py:11-92, differentiated (FP64, on the device:
    d2ic_strain_gl_jvp): G = A^-1 B(u), dE = (dG^T F + F^T dG) / 2 with F = I + G.
    """
    dev = du.device
    u = torch.as_tensor(u, dtype=torch.float64, device=dev).reshape(-1, 2).contiguous()
    X = torch.as_tensor(np.asarray(nodes, dtype=np.float64), device=dev).reshape(-1, 2).contiguous()
    idx = torch.as_tensor(np.ascontiguousarray(np.asarray(nbr_index), dtype=np.int32), device=dev)
    deg = torch.as_tensor(np.ascontiguousarray(np.asarray(nbr_degree), dtype=np.int32), device=dev)
    n = X.shape[0]
    md = int(idx.shape[1]) if idx.ndim == 2 else 0
    dd = du.to(torch.float64).reshape(-1, n, 2).contiguous()
    K = dd.shape[0]
    work = torch.empty(int(_lib.load().d2ic_strain_gl_jvp_work_doubles(n, md)) or 1, dtype=torch.float64, device=dev)
    out = torch.empty((K, n, 3), dtype=torch.float64, device=dev)
    _lib.call("d2ic_strain_gl_jvp", ptr(u), ptr(dd), K, ptr(X), ptr(idx), ptr(deg), n, md, float(gauge_length),
              float(eps), ptr(work), ptr(out), _lib.stream_handle())
    return out.reshape(tuple(du.shape[:-2]) + (n, 3))


class _DICSolveFn(torch.autograd.Function):
    """u* = solve(I2) with the implicit adjoint as backward and jvp."""

    @staticmethod
    def forward(image, holder):
        return holder.forward_solve(image)

    @staticmethod
    def setup_context(ctx, inputs, output):
        ctx.holder = inputs[1]

    @staticmethod
    def backward(ctx, grad_u):
        return ctx.holder.adj.vjp(grad_u[None])[0].to(grad_u.dtype), None

    @staticmethod
    def jvp(ctx, d_image, _):
        return ctx.holder.adj.jvp(d_image[None])[0].to(torch.float32)


class DifferentiableSolve:
    """``u = ds(image)``: the converged solve as a differentiable torch function of the deformed image.

    Forward: the CG engine (the solver's MeshDICConfig) from ``u0``, then
    ``polish`` exact Newton steps; the adjoint is linearised at that point.
    Reverse mode through ``backward()``, forward mode through
    ``torch.autograd.forward_ad`` dual tensors.  ``torch.func`` transforms are
    not supported: their wrapped tensors have no device pointer to hand to the
    kernels.
    """

    def __init__(self, solver, state, u0=None, polish: int = 3, exact: bool = True):
        self.solver, self.state = solver, state
        self.u0 = u0
        self.polish = int(polish)
        self.exact = exact
        self.adj = None

    def forward_solve(self, image):
        st = self.state
        st.u0_nodal = None if self.u0 is None else np.asarray(self.u0, dtype=np.float32)
        img = image.detach().to(torch.float32)
        res = self.solver.solve(st, img)
        u = torch.as_tensor(res.u_nodal, device=img.device)
        if self.polish:
            u = newton_polish(self.solver, st, img, u, st.config.reg_strength, self.polish, self.exact)
        slot = self.solver._ensure(st)
        slot.load_image(img)
        self.adj = ImplicitAdjoint(slot, u, st.config.reg_strength, self.exact)
        return u.clone()

    def __call__(self, image: torch.Tensor) -> torch.Tensor:
        return _DICSolveFn.apply(image, self)
