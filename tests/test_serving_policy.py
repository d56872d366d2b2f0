"""Host logic of the server's size priority (no GPU): which slots the next slice holds.

The policy writes command words through ``DICServer.cmd`` (a device tensor in use); here a plain
list stands in for it, and slots are stand-ins carrying only what the policy reads (the frame's ROI
pixel count and the slice that admitted it).
"""
from __future__ import annotations

from types import SimpleNamespace

from d2ic_gb300 import _lib
from d2ic_gb300.serving import DICServer, ServeConfig


def _server(sizes, admitted_at, slices, hold_pixels=1000, hold_max=3):
    srv = DICServer.__new__(DICServer)                 # no device: only the policy's state
    srv.cfg = ServeConfig(max_slots=len(sizes), hold_pixels=hold_pixels, hold_max_slices=hold_max)
    srv.slots = [None if n is None else (SimpleNamespace(layout=SimpleNamespace(n_pix=n)), None, None, a)
                 for n, a in zip(sizes, admitted_at)]
    srv.cmd = [_lib.CMD_RUN if n is not None else _lib.CMD_IDLE for n in sizes]
    srv.cmd_host = list(srv.cmd)
    srv.held = [0] * len(sizes)
    srv.slices = slices
    return srv


def test_big_frames_sit_out_while_a_small_frame_is_in_flight():
    srv = _server([5000, 200, None, 8000], [0, 1, 0, 2], slices=3)
    srv._apply_holds()
    assert srv.cmd == [_lib.CMD_HOLD, _lib.CMD_RUN, _lib.CMD_IDLE, _lib.CMD_HOLD]
    assert srv.held == [1, 0, 0, 1]


def test_no_small_frame_no_hold_and_new_frames_keep_their_init():
    srv = _server([5000, 8000], [0, 3], slices=3)     # slot 1 admitted for the coming slice
    srv.cmd[1] = srv.cmd_host[1] = _lib.CMD_INIT
    srv._apply_holds()
    assert srv.cmd == [_lib.CMD_RUN, _lib.CMD_INIT]
    srv = _server([5000, 200], [0, 3], slices=3)      # the small frame is new: the big one still waits
    srv.cmd[1] = srv.cmd_host[1] = _lib.CMD_INIT
    srv._apply_holds()
    assert srv.cmd == [_lib.CMD_HOLD, _lib.CMD_INIT]


def test_holds_are_bounded_and_released():
    srv = _server([5000, 200], [0, 0], slices=1, hold_max=2)
    seen = []
    for _ in range(6):
        srv._apply_holds()
        seen.append(srv.cmd[0])
        srv.slices += 1
    H, R = _lib.CMD_HOLD, _lib.CMD_RUN
    assert seen == [H, H, R, H, H, R]                  # never more than hold_max slices in a row
    srv.slots[1] = None                                # the small frame finished
    srv._apply_holds()
    assert srv.cmd[0] == R


def test_policy_off_touches_nothing():
    srv = _server([5000, 200], [0, 0], slices=2, hold_pixels=0)
    srv._apply_holds()
    assert srv.cmd == [_lib.CMD_RUN, _lib.CMD_RUN]
