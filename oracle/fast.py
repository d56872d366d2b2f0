"""ctypes front end of the oracle's C pixel term (oracle/objective_c.c).

Test infrastructure only (see oracle/__init__.py).  Gives the same FP64
objective and gradient as oracle/objective.py (cubic interpolation) fast
enough to run the reference's CG at full benchmark sizes; the tests check the
two agree.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from .cubic import ORACLE_PAD, cubic_sample
from .objective import Problem, cg_solve, reg_energy, reg_energy_grad

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build():
    """Compile the helper with the committed Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle_obj.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.oracle_pixel_terms.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ip, dp, dp,
                                         ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_int]
        L.oracle_pixel_terms.restype = None
        fp = ctypes.POINTER(ctypes.c_float)
        L.oracle_pixel_terms_f32.argtypes = [fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, ip, fp, fp,
                                             ctypes.c_int, fp, ctypes.c_int, ctypes.c_float, dp, fp, ctypes.c_int]
        L.oracle_pixel_terms_f32.restype = None
        _LIB = L
    return _LIB


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


class FastProblem:
    """Cubic-interpolation objective on a :class:`Problem`, pixel term in C.

    ``precision="f64"`` is the oracle.  ``precision="f32"`` runs the same pixel
    arithmetic in float32 (the reference's default x32 precision) and serves
    only as an x32-equivalent CPU timing; the CG control stays in FP64 numpy.
    """

    def __init__(self, pb: Problem, nthreads: int | None = None, precision: str = "f64"):
        assert pb.interpolation == "cubic"
        assert precision in ("f64", "f32")
        self.pb = pb
        self.precision = precision
        dt = np.float64 if precision == "f64" else np.float32
        self.dt = dt
        self.nthreads = nthreads or os.cpu_count() or 1
        self.coeff2 = np.ascontiguousarray(pb.coeff2, dtype=dt)
        self.coords = np.ascontiguousarray(pb.pixel_coords, dtype=dt)
        self.pnodes = np.ascontiguousarray(pb.pixel_nodes, dtype=np.int32)
        self.N = np.ascontiguousarray(pb.pixel_shapeN, dtype=dt)
        self.I1 = np.ascontiguousarray(
            cubic_sample(pb.coeff1, ORACLE_PAD, pb.pixel_coords[:, 0] - 0.5, pb.pixel_coords[:, 1] - 0.5), dtype=dt)
        self.Np = self.coords.shape[0]

    def _pixel(self, u, want_grad):
        dt = self.dt
        u = np.ascontiguousarray(u, dtype=dt)
        Nn = u.shape[0]
        s = ctypes.c_double(0.0)
        denom = max(self.Np, 1)
        g = np.zeros((Nn, 2), dtype=dt) if want_grad else None
        Hc, Wc = self.coeff2.shape
        if self.precision == "f64":
            lib().oracle_pixel_terms(_p(self.coeff2), Hc, Wc, ORACLE_PAD, _p(self.coords),
                                     _p(self.pnodes, ctypes.c_int), _p(self.N), _p(self.I1), self.Np,
                                     _p(u), Nn, 1.0 / denom, ctypes.byref(s),
                                     _p(g) if want_grad else None, self.nthreads)
        else:
            f = ctypes.c_float
            lib().oracle_pixel_terms_f32(_p(self.coeff2, f), Hc, Wc, ORACLE_PAD, _p(self.coords, f),
                                         _p(self.pnodes, ctypes.c_int), _p(self.N, f), _p(self.I1, f), self.Np,
                                         _p(u, f), Nn, 1.0 / denom, ctypes.byref(s),
                                         _p(g, f) if want_grad else None, self.nthreads)
            if g is not None:
                g = g.astype(np.float64)
        return 0.5 * s.value / denom, g

    def value(self, u, alpha_reg):
        Jp, _ = self._pixel(u, False)
        return Jp + alpha_reg * reg_energy(u, self.pb)

    def value_and_grad(self, u, alpha_reg):
        Jp, g = self._pixel(u, True)
        return Jp + alpha_reg * reg_energy(u, self.pb), g + alpha_reg * reg_energy_grad(u, self.pb)

    def cg_solve(self, u0, alpha_reg, max_iter, tol):
        return cg_solve(u0, self.pb, alpha_reg, max_iter, tol,
                        value_and_grad=lambda uu: self.value_and_grad(uu, alpha_reg),
                        value=lambda uu: self.value(uu, alpha_reg))
