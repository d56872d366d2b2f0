"""The C-ABI library loads and exports every symbol declared in include/d2ic_gb300.h (no GPU needed)."""
from __future__ import annotations

import ctypes


def test_library_exports_header_symbols(built_library):
    from d2ic_gb300 import _lib
    names = _lib.header_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(built_library, n)]
    assert not missing, f"symbols declared but not exported: {missing}"
    # every declared symbol has a ctypes signature on the Python side
    assert set(names) <= set(_lib._SIGS)


def test_host_only_entry_points(built_library):
    """Size queries and workspace binding run on the host."""
    from d2ic_gb300 import _lib
    assert built_library.d2ic_version() >= 100
    assert built_library.d2ic_frame_descriptor_bytes() == ctypes.sizeof(_lib.Frame) == 384
    assert _lib.Frame.coeff_map.offset == 0                # the tensor map stays 64-byte aligned
    assert built_library.d2ic_cg_control_bytes(1) > 0
    assert built_library.d2ic_cg_control_bytes(64) > built_library.d2ic_cg_control_bytes(1)
    nb = built_library.d2ic_frame_workspace_bytes(1089, 784, 4)
    assert nb >= 14 * 4 * 1089 + 16 * 4 * 1089 + 40 * 35 + 4 * 36 + 4 * 784
    f = _lib.Frame()
    f.n_nodes, f.n_chunks, f.node_chunk_k = 1089, 784, 4
    fake_ws = 1 << 20                      # never dereferenced: binding only computes addresses
    assert built_library.d2ic_frame_bind_workspace(ctypes.byref(f), fake_ws) == 0
    assert f.node_ws == fake_ws and f.n_groups == 35
    assert f.group_cnt % 256 == 0 and f.node_grad % 256 == 0 and f.group_part % 256 == 0
    assert f.chunk_tile % 256 == 0 and f.chunk_tile + 784 * 4 <= fake_ws + nb
    assert built_library.d2ic_frame_bind_workspace(ctypes.byref(f), fake_ws + 8) == _lib.BAD_ARG
    assert b"256-byte" in built_library.d2ic_last_error_string()


def test_tile_encoding_arguments(built_library):
    """Tile staging: off with width 0, argument checks before any driver call."""
    from d2ic_gb300 import _lib
    f = _lib.Frame()
    f.coeff, f.W, f.H, f.cpitch, f.pad = 1 << 20, 100, 80, 160, 16
    assert built_library.d2ic_frame_encode_tiles(ctypes.byref(f), 0, 0) == 0
    assert f.tile_w == 0 and f.tile_h == 0
    assert built_library.d2ic_frame_encode_tiles(ctypes.byref(f), 30, 24) == _lib.BAD_ARG   # width not /4
    assert built_library.d2ic_frame_encode_tiles(ctypes.byref(f), 64, 24) == _lib.BAD_ARG   # > 736 floats
    f.coeff = (1 << 20) + 4
    assert built_library.d2ic_frame_encode_tiles(ctypes.byref(f), 28, 24) == _lib.BAD_ARG   # misaligned base
    assert f.tile_w == 0
