"""ctypes binding of libd2ic_gb300.so (the C ABI declared in include/d2ic_gb300.h).

The library is loaded from the package's in-tree ``_build`` directory.  There
is no fallback: if the library is missing, the first GPU call raises.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libd2ic_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "d2ic_gb300.h")

OK = 0
BAD_ARG = -1
OOM = -2
NAN_DETECTED = -3
MAX_ITERS = -4
WAIT_TIMEOUT = -5
CUDA_ERROR = -6
UNSUPPORTED = -7
INTERNAL = -8
RUNNING = 1
CMD_INIT, CMD_RUN, CMD_IDLE, CMD_HOLD = 0, 1, 2, 3
STOP_ON_FINISH, STOP_ON_IRQ = 1, 2

INTERP_CUBIC = 0
INTERP_LINEAR = 1
NODE_GROUP = 32
NPART = 5
MAX_FRAMES = 4096
CHUNK_MAX = 256
TILE_MAX_FLOATS = 736

STATUS_NAMES = {OK: "ok", BAD_ARG: "bad_arg", OOM: "oom", NAN_DETECTED: "nan_detected",
                MAX_ITERS: "max_iters", WAIT_TIMEOUT: "wait_timeout", CUDA_ERROR: "cuda_error",
                UNSUPPORTED: "unsupported", INTERNAL: "internal", RUNNING: "running"}

vp = ctypes.c_void_p
i32 = ctypes.c_int
f32 = ctypes.c_float
f64 = ctypes.c_double
szt = ctypes.c_size_t


class Frame(ctypes.Structure):
    """Mirror of ``d2ic_frame_t``."""
    _fields_ = [
        ("coeff_map", ctypes.c_uint64 * 16),
        ("coeff", vp), ("pix", vp), ("chunk_begin", vp), ("chunk_nodes", vp),
        ("chunk_box", vp), ("chunk_slot", vp), ("group_need", vp), ("nbr_index", vp), ("nbr_weight", vp),
        ("u0", vp), ("u_out", vp), ("hist", vp), ("n_iters", vp), ("status", vp), ("n_evals", vp),
        ("node_ws", vp), ("node_grad", vp), ("group_part", vp), ("group_cnt", vp), ("chunk_tile", vp),
        ("tol", f64), ("alpha_reg", f32), ("max_iter", i32),
        ("W", i32), ("H", i32), ("cpitch", i32), ("pad", i32),
        ("n_pix", i32), ("n_chunks", i32), ("n_nodes", i32), ("max_deg", i32),
        ("n_groups", i32), ("node_chunk_k", i32), ("tile_w", i32), ("tile_h", i32), ("reserved_", i32 * 8),
    ]


class Grid(ctypes.Structure):
    """d2ic_grid_t: a tensor-grid mesh and ROI mask on the device (include/d2ic_gb300.h)."""
    _fields_ = [
        ("gx", vp), ("gy", vp), ("nx", i32), ("ny", i32), ("cell", vp), ("elem_cell", vp), ("elements", vp),
        ("nodes", vp), ("roi", vp), ("n_elem", i32), ("n_nodes", i32), ("H", i32), ("W", i32),
        ("i0", i32), ("i1", i32), ("j0", i32), ("j1", i32),
    ]


_SIGS = {
    "d2ic_last_error_string": (ctypes.c_char_p, []),
    "d2ic_version": (i32, []),
    "d2ic_frame_descriptor_bytes": (szt, []),
    "d2ic_device_info": (i32, [i32, vp, vp]),
    "d2ic_bspline_prefilter": (i32, [vp, i32, i32, i32, i32, vp, vp, vp]),
    "d2ic_bspline_prefilter_batch": (i32, [vp, i32, i32, i32, i32, i32, vp, vp, vp]),
    "d2ic_pad_image": (i32, [vp, i32, i32, i32, i32, vp, vp]),
    "d2ic_bspline_prefilter_u8": (i32, [vp, i32, i32, i32, i32, vp, vp, vp]),
    "d2ic_pad_image_u8": (i32, [vp, i32, i32, i32, i32, vp, vp]),
    "d2ic_render_speckle": (i32, [vp, vp, f32, i32, i32, f32, vp, i32, i32, vp, vp]),
    "d2ic_speckle_finish": (i32, [vp, ctypes.c_longlong, f32, f32, f32, ctypes.c_ulonglong, i32, vp, vp]),
    "d2ic_sample_points": (i32, [vp, i32, i32, i32, i32, i32, vp, i32, vp, vp, vp, vp]),
    "d2ic_pack_pixels": (i32, [vp, vp, i32, vp, i32, i32, i32, i32, i32, vp, vp]),
    "d2ic_frame_workspace_bytes": (szt, [i32, i32, i32]),
    "d2ic_frame_bind_workspace": (i32, [vp, vp]),
    "d2ic_frame_encode_tiles": (i32, [vp, i32, i32]),
    "d2ic_cg_control_bytes": (szt, [i32]),
    "d2ic_cg_solve_batched": (i32, [vp, i32, vp, szt, i32, i32, vp]),
    "d2ic_cg_solve_traced": (i32, [vp, i32, vp, szt, i32, i32, vp, i32, vp]),
    "d2ic_cg_solve_noalloc": (i32, [vp, i32, vp]),
    "d2ic_cg_command_offset": (szt, []),
    "d2ic_cg_slice": (i32, [vp, i32, vp, szt, i32, i32, i32, vp]),
    "d2ic_cg_slice_ex": (i32, [vp, i32, vp, szt, i32, i32, i32, i32, vp]),
    "d2ic_cg_irq_offset": (szt, []),
    "d2ic_eval_objective": (i32, [vp, vp, vp, szt, i32, vp, vp, vp]),
    "d2ic_hessian_chunks": (i32, [vp, i32, vp, i32, vp, vp]),
    "d2ic_hessian_matvec": (i32, [vp, i32, i32, vp, vp, i32, f32, f32, vp, vp, vp]),
    "d2ic_hessian_op_bytes": (szt, [i32, i32]),
    "d2ic_hessian_assemble": (i32, [vp, i32, i32, i32, vp, f32, f32, vp, szt, vp]),
    "d2ic_hessian_apply": (i32, [vp, i32, i32, vp, i32, vp, vp]),
    "d2ic_mixed_term": (i32, [vp, i32, i32, vp, vp, f32, vp, vp, i32, i32, vp]),
    "d2ic_mixed_term_batch": (i32, [vp, i32, i32, i32, vp, vp, i32, ctypes.c_longlong, f32, vp, vp, i32, i32, vp]),
    "d2ic_mixed_term_T": (i32, [vp, i32, vp, vp, f32, vp, vp]),
    "d2ic_bspline_prefilter_T": (i32, [vp, i32, i32, i32, i32, vp, vp, vp]),
    "d2ic_zncc_match":(i32, [vp, i32, i32, vp, i32, i32, vp, i32, i32, i32, vp, vp, vp]),
    "d2ic_idw_project": (i32, [vp, i32, vp, vp, i32, f32, vp, vp]),
    "d2ic_strain_gl": (i32, [vp, vp, vp, vp, i32, i32, f32, f32, vp, vp, vp]),
    "d2ic_strain_gl_jvp_work_doubles": (szt, [i32, i32]),
    "d2ic_strain_gl_jvp": (i32, [vp, vp, i32, vp, vp, vp, i32, i32, f64, f64, vp, vp, vp]),
    "d2ic_discrepancy_map": (i32, [vp, i32, vp, vp, vp, i32, i32, vp, vp, vp, vp]),
    "d2ic_central_gradient": (i32, [vp, i32, i32, vp, vp, vp]),
    "d2ic_local_coordinates": (i32, [vp, vp, vp, ctypes.c_longlong, i32, vp, vp, vp]),
    "d2ic_grid_count": (i32, [vp, vp, vp]),
    "d2ic_grid_scratch_bytes": (szt, [ctypes.c_longlong, i32]),
    "d2ic_grid_layout": (i32, [vp, vp, vp, ctypes.c_longlong, i32, i32, vp, i32, i32, vp, szt, vp, vp, vp, vp, vp, vp,
                               vp, vp]),
    "d2ic_grid_springs": (i32, [vp, vp, i32, vp, vp, vp]),
    "d2ic_structured_assign": (i32, [vp, ctypes.c_longlong, vp, i32, vp, i32, vp, vp, vp]),
    "d2ic_pcg_work_bytes": (szt, [i32, i32, i32]),
    "d2ic_pcg_solve": (i32, [vp, i32, i32, i32, vp, f32, f32, vp, vp, vp, vp, i32, f64, i32, vp, szt, vp, vp]),
    "d2ic_local_gn_slot_bytes": (szt, [i32, i32]),
    "d2ic_local_gn_sweep": (i32, [vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, i32, vp, f32, f32, f32,
                                  f32, vp, vp, vp]),
}

_lib = None


class D2ICError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{STATUS_NAMES.get(code, code)}] {msg}")
        self.code = code


def header_symbols() -> list[str]:
    """Function names declared in include/d2ic_gb300.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^D2IC_API\s+[\w\s\*]+?\b(d2ic_\w+)\s*\(", txt, flags=re.M)))


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"d2ic_gb300 CUDA library not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or `python -m d2ic_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(code: int):
    """Raise the Python exception matching a C status (ValueError for bad arguments)."""
    if code == OK:
        return
    msg = load().d2ic_last_error_string().decode(errors="replace")
    if code == BAD_ARG:
        raise ValueError(msg)
    if code == OOM:
        raise MemoryError(msg)
    raise D2ICError(code, msg)


def call(name: str, *args):
    check(getattr(load(), name)(*args))


def ptr(t) -> int:
    """Device (or host) address of a torch tensor / numpy array, or 0 for None."""
    if t is None:
        return 0
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def stream_handle(stream=None) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
