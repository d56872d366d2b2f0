#!/usr/bin/env python
"""Benchmark of the global FE-DIC hot path on GB300.

Workload (default ``plate_hole_2048``): 2048^2 synthetic speckle, 1800^2
square minus an r = 300 disk, 16 px Q4 elements (16,641 nodes, 2.92 M ROI
pixels), 20 frames of the plate-hole field; frame 0 initialised by ZNCC +
IDW, later frames warm-started from the previous solution; CG tol 1e-3,
reg 0.1, max 200 iterations.  One step = the whole 20-frame sequence.

* ``value``: frames/s with the images already in HBM (device-resident
  sequence path), L2 flushed (256 MB write) between steps;
* ``e2e``: the same frames/s through the public API (DICInitMotion for frame
  0, then BatchMeshBased.run) from pinned host frames, per-frame device->host
  results included; per-frame p50/p99 latency reported beside it;
* ``roofline``: the persistent CG kernel's algorithmic bytes (48 B per ROI
  pixel and 128 B per node per objective evaluation) over its CUDA-event
  duration, against the measured HBM copy bandwidth;
* ``cpu_baseline``: the FP64 oracle restatement (C, OpenMP) on the host cores
  over a bounded sample of the same sequence.

``--impl reference`` times that CPU restatement alone (the reference itself is
JAX and cannot be installed offline).  Multi-GPU: one independent replica
sequence per rank (frames shard by sequence, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

B_PIX = 48      # algorithmic bytes per ROI pixel per objective evaluation
B_NODE = 128    # spring matvec (80) + CG vector ops (48) per node per evaluation


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", default="plate_hole_2048",
                   choices=["plate_hole_2048", "plate_hole_4096", "translation_512"])
    p.add_argument("--frames", type=int, default=20)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-sample-frames", type=int, default=2)
    p.add_argument("--no-serve", action="store_true", help="skip the 512^2 small-frame serving stream")
    p.add_argument("--serve-mixed", action="store_true", help="also run the reduced mixed serving stream")
    p.add_argument("--serve-seqs", type=int, default=16)
    p.add_argument("--serve-frames", type=int, default=4)
    p.add_argument("--serve-slots", type=int, default=32)
    p.add_argument("--serve-slice", type=int, default=16)
    p.add_argument("--no-4096", action="store_true", help="skip the 4096^2 engine measurement")
    p.add_argument("--frames-4096", type=int, default=3)
    p.add_argument("--no-stream", action="store_true", help="skip the serving stream")
    p.add_argument("--stream-frames", type=int, default=4096)
    p.add_argument("--stream-seqs", type=int, default=128)
    p.add_argument("--stream-plain-frames", type=int, default=4096)
    p.add_argument("--stream-hold-pixels", type=int, default=5_000_000,
                   help="serving stream: size priority threshold in ROI pixels (ServeConfig.hold_pixels; "
                        "the 4096^2 frames sit out slices while smaller frames are in flight; 0: off)")
    p.add_argument("--stream-slots", type=int, default=64,
                   help="frames in flight in the server (the engine keeps up to 64 active frames' lookup "
                        "tables in shared memory)")
    p.add_argument("--stream-rates", type=lambda v: [float(x) for x in v.split(",")],
                   default=[50.0, 100.0, 200.0, 500.0, 1000.0, 2000.0])
    p.add_argument("--stream-window", type=float, default=20.0,
                   help="arrivals per rate: the whole stream, or at least 1024 and about this many seconds")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--batch-frames", type=int, default=64)
    p.add_argument("--batch-sides", default="512,1024,2048,3072,4096",
                   help="image sides drawn for the uneven batch")
    p.add_argument("--no-local", action="store_true")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--adjoint-realisations", type=int, default=256)
    p.add_argument("--adjoint-fd-dirs", type=int, default=32)
    return p.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return ws, rank, local


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def make_workload(name: str, n_frames: int, seed: int, device):
    from d2ic_gb300 import workloads
    if name == "plate_hole_2048":
        return workloads.plate_hole_2048(n_frames=n_frames, seed=seed, device=device)
    if name == "plate_hole_4096":     # same field scaled to 4096^2: pixel data larger than L2 (profiling case)
        return workloads.plate_hole_2048(n_frames=n_frames, seed=seed, device=device, H=4096)
    return workloads.translation_512(seed=seed, device=device)


# ---------------------------------------------------------------------------
# CPU restatement (oracle) leg
# ---------------------------------------------------------------------------

def cpu_sequence_sample(wl, n_sample: int, u_start=None):
    """Time the FP64 oracle (C pixel term, OpenMP on all host cores) on frames 1..n_sample."""
    from oracle import fast, objective, pixels
    H, W = wl.ref.shape
    oa = pixels.build_pixel_assets(np.asarray(wl.mesh.nodes_xy), np.asarray(wl.mesh.elements), H, W,
                                   wl.assets.roi_mask)
    cfg = wl.config
    frames = list(range(1, min(n_sample, len(wl.frames) - 1) + 1)) if len(wl.frames) > 1 else [0]
    u = np.zeros((wl.n_nodes, 2)) if u_start is None else np.asarray(u_start, np.float64)
    t_solve = 0.0
    iters = []
    sols = {}
    for k in frames:
        pb = objective.Problem.build(wl.ref, wl.frames[k], oa)        # coefficients: setup, not timed
        fp = fast.FastProblem(pb)
        t0 = time.perf_counter()
        u, h, kk, ne = fp.cg_solve(u, cfg.reg_strength, cfg.max_iters, cfg.tol)
        t_solve += time.perf_counter() - t0
        iters.append(int(kk))
        sols[k] = (u.copy(), int(kk))
    cores = os.cpu_count() or 1
    return {"value": len(frames) / t_solve, "unit": "frames/s", "cores": cores, "kind": "port",
            "sample": f"{wl.name}: frames {frames[0]}..{frames[-1]} warm-started, FP64 C oracle CG "
                      f"({cores} OpenMP threads), {sum(iters)} iterations in {t_solve:.1f} s"}, sols


def parity_block(wl, res, sols):
    """GPU frames against the FP64 oracle's solves of the same frames from the same start (frame 0's
    GPU solution), over the used nodes; plus how many of the sequence's frames hit max_iters."""
    used = np.unique(np.asarray(wl.mesh.elements))
    u_gpu = res.u.cpu().numpy().astype(np.float64)
    info = res.info.cpu().numpy()
    per = []
    for k, (ur, kr) in sorted(sols.items()):
        d = np.abs(u_gpu[k][used] - ur[used]).max(axis=1)
        per.append({"frame": int(k), "max_err_px": float(d.max()), "mean_err_px": float(d.mean()),
                    "gpu_iters": int(info[k, 0]), "oracle_iters": int(kr)})
    capped = int(np.sum(info[:, 0] >= wl.config.max_iters))
    return {"reference": "FP64 oracle (C pixel term), same frames, warm-started from the GPU's frame-0 solution",
            "frames": per, "max_err_px": max(p["max_err_px"] for p in per) if per else None,
            "mean_err_px": float(np.mean([p["mean_err_px"] for p in per])) if per else None,
            "same_iterations": all(p["gpu_iters"] == p["oracle_iters"] for p in per),
            "frames_at_max_iters": capped, "frames_in_sequence": int(info.shape[0]),
            "max_iters": int(wl.config.max_iters), "tolerance_px": 1e-3}


def reference_workload(name: str, n_frames: int, seed: int):
    """The workload built on the host alone for the CPU arm: speckle synthesis in CPU torch (same
    seeds as the GPU arm), mesh and pixel assets from the oracle's restatement of the reference's
    mesher and asset builder.  Nothing of the CUDA library is loaded."""
    from d2ic_gb300.synthetic import PlateHoleField, Translation, plate_hole_mask, rect_mask, speckle_sequence
    from oracle import mesh as omesh
    from oracle import pixels
    if name.startswith("plate_hole"):
        H = 2048 if name == "plate_hole_2048" else 4096
        s = H / 2048.0
        warps = [PlateHoleField(k / 19.0, cx=1024 * s, cy=1024 * s, L=2048 * s) for k in range(n_frames)]
        ref, frames = speckle_sequence(H, H, warps, seed=seed, noise_seeds=[seed] + [100 + k for k in range(n_frames)],
                                       device="cpu")
        mask = plate_hole_mask(H, H, int(round(1800 * s)), 300.0 * s)
        elem, init = 16, (17, 8, 0.2)
    else:
        H = 512
        ref, frames = speckle_sequence(H, H, [Translation(0.35, -0.62)], seed=seed, noise_seeds=[seed, seed + 1],
                                       device="cpu")
        mask = rect_mask(H, H, 448, 448)
        elem, init = 16, None
    m = omesh.mask_to_mesh_assets(mask, elem)
    oa = pixels.build_pixel_assets(m["nodes"], m["elements"], H, H, m["roi_mask"])
    return {"name": name, "ref": ref, "frames": frames, "mesh": m, "assets": oa, "init": init,
            "max_iters": 200, "tol": 1e-3, "reg": 0.1}


def reference_sequence(wl, precision: str):
    """The reference's sequence path on the CPU (oracle restatement): frame 0 from ZNCC at element
    centres + IDW, every later frame warm-started from the previous solution, nonlinear CG per
    frame.  Returns (seconds, CG iterations per frame); image coefficients are set-up, not timed."""
    from oracle import fast, init_motion, objective
    m = wl["mesh"]
    probs = [fast.FastProblem(objective.Problem.build(wl["ref"], f, wl["assets"]), precision=precision)
             for f in wl["frames"]]
    t0 = time.perf_counter()
    if wl["init"] is not None:
        win, search, smin = wl["init"]
        uc, sc = init_motion.match_centers(m["centers"], wl["ref"], wl["frames"][0], win, search)
        uc, _ = init_motion.apply_score_min(uc, sc, smin)
        u = init_motion.project_centers_to_nodes_idw(m["nodes"], m["centers"], uc)
    else:
        u = np.zeros_like(m["nodes"])
    iters = []
    for fp in probs:
        u, _, k, _ = fp.cg_solve(u, wl["reg"], wl["max_iters"], wl["tol"])
        iters.append(int(k))
    return time.perf_counter() - t0, iters


def run_reference(args, ws, rank):
    """CPU arm: the reference's algorithm on the host cores (its JAX code cannot be installed here),
    timed on a bounded sample of the GPU arm's sequence: frames 0..n of the same workload."""
    if rank != 0:
        return
    n = max(1, min(args.frames, 1 + args.cpu_sample_frames))
    t0 = time.perf_counter()
    wl = reference_workload(args.workload, n, 1)
    n = len(wl["frames"])
    t_setup = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    vals, iters32 = [], None
    for _ in range(max(1, min(args.steps, 2))):          # each step is a 10-30 s sample
        t, iters32 = reference_sequence(wl, "f32")
        vals.append(n / t)
    t64, iters64 = reference_sequence(wl, "f64")
    v = statistics.median(vals)
    sample = (f"{wl['name']}: frames 0..{n - 1} of the GPU arm's sequence (ZNCC + IDW start, then warm-started "
              f"CG), C pixel term on {cores} OpenMP threads, CG control in numpy")
    line = {"metric": "frames/s", "value": v, "unit": "frames/s", "n_gpus": args.gpus, "steps": len(vals),
            "warmup": 0, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (x32-equivalent; f64 beside it)", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": wl["name"], "frames": args.frames, "sample_frames": n,
                       "image": list(wl["ref"].shape), "roi_pixels": int(wl["assets"]["pixel_coords_ref"].shape[0]),
                       "nodes": int(wl["mesh"]["nodes"].shape[0]), "max_iters": wl["max_iters"], "tol": wl["tol"],
                       "reg": wl["reg"]},
            "cpu_baseline": {"value": v, "unit": "frames/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cg_iterations": {"f32": iters32, "f64": iters64},
            "f64": {"value": n / t64, "unit": "frames/s", "seconds": t64},
            "setup_s": round(t_setup, 1),
            "note": "the reference is JAX: its offline install fails on dm-pix and, with --no-deps, it does not "
                    "import (no jax), so this arm times the oracle's restatement of its sequence path (ZNCC + IDW "
                    "initial motion, warm-started nonlinear CG) on the host cores only; value = float32 pixel "
                    "arithmetic, the reference's default x32 precision; f64 = the FP64 oracle"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# served vs plain on a mixed stream
# ---------------------------------------------------------------------------

def run_serving(args, dev, sides=(512, 1024, 2048), n_seq=None, label="mixed_stream"):
    """Plain single-frame drop-in vs the continuous-batching server on the same requests."""
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300 import workloads
    from d2ic_gb300.serving import DICServer, Request, ServeConfig

    seqs = workloads.mixed_stream(n_seq=n_seq or args.serve_seqs, frames_per_seq=args.serve_frames, device=dev,
                                  sides=tuple(sides))
    F = args.serve_frames
    order = [(s, k) for k in range(F) for s in range(len(seqs))]
    pinned = [[torch.from_numpy(f).pin_memory() for f in wl.frames] for wl in seqs]
    n_pix = sum(wl.n_pix for wl in seqs) * F

    # plain: the reference's per-frame pipeline on our drop-in (one launch + host sync per frame)
    dics, inits = [], []
    for wl in seqs:
        dic = d2.DICMeshBased(wl.mesh, d2.GlobalCGSolver(device=dev), wl.config)
        dic.prepare(wl.ref, wl.assets)
        ini = d2.DICInitMotion(wl.init, d2.TranslationZNCCSolver(wl.init, device=dev))
        ini.prepare(wl.ref, dic.state.assets)
        dics.append(dic)
        inits.append(ini)

    def plain_pass():
        prev = [None] * len(seqs)
        out, lat = {}, []
        for s, k in order:
            t0 = time.perf_counter()
            if k == 0:
                dics[s].set_initial_guess(inits[s].run(pinned[s][0]).u_nodal)
            else:
                dics[s].set_initial_guess(prev[s])
            r = dics[s].run(pinned[s][k])
            prev[s] = r.u_nodal
            out[(s, k)] = np.asarray(r.u_nodal)
            lat.append(time.perf_counter() - t0)
        return out, lat

    plain_pass()                                         # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_u, plain_lat = plain_pass()
    t_plain = time.perf_counter() - t0

    srv = DICServer(dev, ServeConfig(max_slots=args.serve_slots, slice_rounds=args.serve_slice, autotune=True))
    for s, wl in enumerate(seqs):
        srv.add_sequence(s, wl.ref, wl.mesh, wl.assets, wl.config, init=wl.init)

    def served_pass(offsets=None):
        srv.reset_sequences()
        reqs = [Request(s, k, pinned[s][k]) for s, k in order]
        if offsets is None:
            t = time.perf_counter()
            for r in reqs:
                r.t_arrival = t
                srv.submit(r)
            srv.run_until_idle()
        else:
            srv.run_stream(reqs, offsets)
        return reqs

    served_pass()                                        # warm-up (graph capture)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reqs = served_pass()
    t_served = time.perf_counter() - t0
    diff = max(float(np.abs(r.u - plain_u[(r.seq_id, r.frame_index)]).max()) for r in reqs)
    served_fps = len(reqs) / t_served
    # online: Poisson arrivals at fractions of the measured served throughput (rate sweep)
    sweep = []
    for frac in (0.25, 0.5, 0.75, 1.0):
        rate_k = frac * served_fps
        rng = np.random.default_rng(4)
        offs = np.cumsum(rng.exponential(1.0 / rate_k, len(order)))
        t_on = time.perf_counter()
        reqs_k = served_pass(offs)
        wall = time.perf_counter() - t_on
        lat_k = np.array([r.latency for r in reqs_k])
        plain_k = _fifo_latency(offs, plain_lat)         # the plain form at the same arrivals
        sweep.append({"offered_frames_per_s": rate_k, "achieved_frames_per_s": len(reqs_k) / wall,
                      "latency_ms_p50": 1000 * float(np.percentile(lat_k, 50)),
                      "latency_ms_p99": 1000 * float(np.percentile(lat_k, 99)),
                      "plain_latency_ms_p50": 1000 * float(np.percentile(plain_k, 50)),
                      "plain_latency_ms_p99": 1000 * float(np.percentile(plain_k, 99))})
    rate = sweep[1]["offered_frames_per_s"]
    lat = None
    return {"workload": label, "sequences": len(seqs), "frames": len(order),
            "image_sides": sorted({int(wl.ref.shape[0]) for wl in seqs}), "roi_pixels_per_pass": int(n_pix),
            "plain_frames_per_s": len(order) / t_plain, "served_frames_per_s": served_fps,
            "speedup": served_fps / (len(order) / t_plain), "max_abs_diff_vs_plain_px": diff,
            "plain_latency_ms_p50": 1000 * float(np.percentile(plain_lat, 50)),
            "plain_latency_ms_p99": 1000 * float(np.percentile(plain_lat, 99)),
            "online_rate_frames_per_s": rate, "latency_ms_p50": sweep[1]["latency_ms_p50"],
            "latency_ms_p99": sweep[1]["latency_ms_p99"], "rate_sweep": sweep, "slots": args.serve_slots,
            "slice_rounds": args.serve_slice, "graphs": sorted(srv.graphs)}


# ---------------------------------------------------------------------------
# the serving stream: Poisson arrivals from many concurrent sequences
# ---------------------------------------------------------------------------

def _fifo_latency(arrivals, service):
    """Latencies of a single first-come-first-served server (the plain drop-in handles one frame at
    a time): frame i starts at max(arrival_i, end of frame i-1) and takes service_i."""
    t_free, out = 0.0, []
    for a, sv in zip(arrivals, service):
        t0 = max(a, t_free)
        t_free = t0 + sv
        out.append(t_free - a)
    return np.asarray(out)


def _stream_parity(stream, done, n_check=3):
    """Served frames against FP64 oracle solves of the same frame from the same warm start (the
    served result of the sequence's previous frame), on the smallest sequences."""
    from oracle import fast, objective, pixels
    out = []
    seqs = sorted(stream.sequences, key=lambda q: (q.side, -q.element_px))
    for q in seqs:
        if len(out) >= n_check:
            break
        if (q.seq_id, 1) not in done or (q.seq_id, 0) not in done:
            continue
        H = q.side
        oa = pixels.build_pixel_assets(np.asarray(q.mesh.nodes_xy), np.asarray(q.mesh.elements), H, H,
                                       q.assets.roi_mask)
        pb = objective.Problem.build(q.ref.astype(np.float64), q.frames[1].numpy().astype(np.float64), oa)
        u0 = done[(q.seq_id, 0)].u.astype(np.float64)
        ur, _, kr, _ = fast.FastProblem(pb).cg_solve(u0, q.config.reg_strength, q.config.max_iters, q.config.tol)
        r = done[(q.seq_id, 1)]
        used = np.unique(np.asarray(q.mesh.elements))
        out.append({"sequence": q.seq_id, "side": H, "element_px": q.element_px, "frame": 1,
                    "max_err_px": float(np.abs(r.u[used] - ur[used]).max()), "gpu_iters": int(r.n_iters),
                    "oracle_iters": int(kr)})
    return out


def run_serving_stream(args, dev):
    """Plain single-frame drop-in vs the continuous-batching server on the serving stream: 4096
    Poisson arrivals from 128 sequences (sides 512-4096, elements 8-32 px), swept over offered
    rates; frames are 8-bit camera images in pinned host memory."""
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300 import workloads
    from d2ic_gb300.serving import DICServer, Request, ServeConfig

    t0 = time.perf_counter()
    st = workloads.serving_stream(n_arrivals=args.stream_frames, n_seq=args.stream_seqs, device=dev)
    t_build = time.perf_counter() - t0
    seqs = st.sequences
    N = len(st.order)
    roi = {q.seq_id: q.assets.pixel_data.n_pixels for q in seqs}

    # plain drop-in: one DICMeshBased per sequence, frames one at a time in arrival order
    t0 = time.perf_counter()
    dics, inits = {}, {}
    for q in seqs:
        dic = d2.DICMeshBased(q.mesh, d2.GlobalCGSolver(device=dev), q.config)
        dic.prepare(q.ref, q.assets)
        ini = d2.DICInitMotion(q.init, d2.TranslationZNCCSolver(q.init, device=dev))
        ini.prepare(q.ref, dic.state.assets)
        dics[q.seq_id], inits[q.seq_id] = dic, ini
    t_plain_setup = time.perf_counter() - t0

    def plain(order):
        prev, svc, out = {}, [], {}
        for s, k in order:
            t = time.perf_counter()
            img = seqs[s].frames[k]
            dics[s].set_initial_guess(inits[s].run(img).u_nodal if k == 0 else prev[s])
            r = dics[s].run(img)
            prev[s] = r.u_nodal
            svc.append(time.perf_counter() - t)
            out[(s, k)] = np.asarray(r.u_nodal)
        return svc, out

    n_plain = min(N, args.stream_plain_frames)
    plain([(q.seq_id, 0) for q in seqs[:8]])                      # warm-up (lazy device buffers)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    svc, plain_u = plain(st.order[:n_plain])
    t_plain = time.perf_counter() - t0
    plain_fps = n_plain / t_plain

    t0 = time.perf_counter()
    srv = DICServer(dev, ServeConfig(max_slots=min(len(seqs), args.stream_slots), slice_rounds=args.serve_slice,
                                     hold_pixels=args.stream_hold_pixels))
    for q in seqs:
        srv.add_sequence(q.seq_id, q.ref, q.mesh, q.assets, q.config, init=q.init)
    t_srv_setup = time.perf_counter() - t0

    def served(n, offsets=None):
        srv.reset_sequences()
        reqs = [Request(s, k, seqs[s].frames[k]) for s, k in st.order[:n]]
        t = time.perf_counter()
        if offsets is None:
            for r in reqs:
                r.t_arrival = t
                srv.submit(r)
            srv.run_until_idle()
        else:
            srv.run_stream(reqs, offsets)
        return reqs, time.perf_counter() - t

    served(min(N, 256))                                           # warm-up: graph capture
    torch.cuda.synchronize()
    reqs, t_sat = served(N)
    served_fps = N / t_sat
    done = {(r.seq_id, r.frame_index): r for r in reqs}
    diffs = {key: float(np.abs(done[key].u - u).max()) for key, u in plain_u.items()}
    diff = max(diffs.values())
    side_of = {q.seq_id: q.side for q in seqs}
    svc_by_side, svc_by_elem = {}, {}
    elem_of = {q.seq_id: q.element_px for q in seqs}
    for (s_id, _k), t in zip(st.order[:n_plain], svc):
        svc_by_side.setdefault(side_of[s_id], []).append(t)
        svc_by_elem.setdefault((side_of[s_id], elem_of[s_id]), []).append(t)
    it_capped = sum(1 for r in reqs if r.n_iters is not None and r.n_iters >= seqs[r.seq_id].config.max_iters)
    sweep = []
    for rate in args.stream_rates:
        n = min(N, max(1024, int(args.stream_window * rate)))
        offs = st.offsets(rate, n)
        reqs_k, wall = served(n, offs)
        lat = np.array([r.latency for r in reqs_k])
        plain_lat = _fifo_latency(offs[:min(n, n_plain)], svc[:min(n, n_plain)])
        sweep.append({"offered_frames_per_s": rate, "arrivals": n, "achieved_frames_per_s": n / wall,
                      "latency_ms_p50": 1000 * float(np.percentile(lat, 50)),
                      "latency_ms_p99": 1000 * float(np.percentile(lat, 99)),
                      "plain_latency_ms_p50": 1000 * float(np.percentile(plain_lat, 50)),
                      "plain_latency_ms_p99": 1000 * float(np.percentile(plain_lat, 99)),
                      "plain_latency_arrivals": int(len(plain_lat))})
    parity = _stream_parity(st, done)
    by_side = {}
    for q in seqs:
        by_side.setdefault(q.side, []).append(q.seq_id)
    return {"workload": "serving_stream", "arrivals": N, "sequences": len(seqs),
            "image_sides": sorted(by_side), "element_px": sorted({q.element_px for q in seqs}),
            "sequences_per_side": {str(k): len(v) for k, v in sorted(by_side.items())},
            "roi_pixels_per_pass": int(sum(roi[s] for s, _ in st.order)), "frame_dtype": "uint8",
            "host_frame_bytes": st.host_bytes,
            "plain_frames_per_s": plain_fps, "plain_frames_timed": n_plain,
            "plain_service_ms_p50": 1000 * float(np.percentile(svc, 50)),
            "served_frames_per_s": served_fps, "speedup": served_fps / plain_fps,
            "max_abs_diff_vs_plain_px": diff,
            "frames_differing_from_plain": int(sum(v > 0 for v in diffs.values())),
            "max_abs_diff_vs_plain_first_frames_px": max([v for (s_id, k), v in diffs.items() if k == 0], default=0.0),
            "plain_service_ms_p50_by_side": {str(k): 1000 * float(np.percentile(v, 50))
                                             for k, v in sorted(svc_by_side.items())},
            "plain_seconds_by_side": {str(k): float(np.sum(v)) for k, v in sorted(svc_by_side.items())},
            "plain_service_ms_p50_by_side_and_element": {f"{a}px_e{b}": 1000 * float(np.percentile(v, 50))
                                                         for (a, b), v in sorted(svc_by_elem.items())},
            "frames_at_max_iters": it_capped,
            "rate_sweep": sweep, "parity_sampled": parity, "slots": min(len(seqs), args.stream_slots),
            "hold_pixels": args.stream_hold_pixels,
            "slice_rounds": args.serve_slice, "graphs": sorted(srv.graphs), "long_slices": srv.long_slices,
            "setup_s": {"stream": round(t_build, 1), "plain": round(t_plain_setup, 1),
                        "server": round(t_srv_setup, 1)},
            "notes": "plain latency per rate: a first-come-first-served queue over the plain drop-in's measured "
                     "per-frame service times (it solves one frame at a time); served latency measured live"}


# ---------------------------------------------------------------------------
# uneven frames in one persistent launch
# ---------------------------------------------------------------------------

def run_batched(args, dev):
    """64 independent frames of uneven size: one batched launch vs one launch per frame."""
    import torch

    from d2ic_gb300 import workloads
    from d2ic_gb300.autotune import default_tuner
    from d2ic_gb300.engine import Engine, FrameLayout, FrameSlot, as_device_image, descriptors_to_device

    sides = tuple(int(x) for x in args.batch_sides.split(","))
    t0 = time.perf_counter()
    wls = workloads.uneven_batch(args.batch_frames, device=dev, sides=sides, device_assets=True)
    t_assets = time.perf_counter() - t0
    tuner = default_tuner(dev)
    slots, shapes = [], []
    t0 = time.perf_counter()
    for wl in wls:
        ref = as_device_image(wl.ref, dev)
        shape = tuner.tune(wl.assets.pixel_data, wl.n_nodes, ref, torch.roll(ref, 1, dims=1), "cubic")
        shapes.append(shape.chunk_pixels)
        lay = FrameLayout(wl.assets.pixel_data, wl.n_nodes, wl.ref, "cubic", dev, chunk_max=shape.chunk_pixels)
        sl = FrameSlot(lay, wl.config.max_iters)
        sl.set_params(wl.config.tol, wl.config.reg_strength)
        sl.load_image(wl.frames[0])
        sl.set_u0(None)
        slots.append(sl)
    t_tune = time.perf_counter() - t0
    n = len(slots)
    desc_all = descriptors_to_device([s.desc for s in slots], dev)
    desc_one = [descriptors_to_device([s.desc], dev) for s in slots]
    eng = Engine(dev, n)
    eng1 = Engine(dev, 1)

    def batched():
        eng.solve(desc_all, n, slots[0].layout.kind)

    def one_by_one():
        for d in desc_one:
            eng1.solve(d, 1, slots[0].layout.kind)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1000.0)
        return statistics.median(ts)

    t_one = timed(one_by_one, max(1, args.steps))
    u_one = [s.u_out.clone() for s in slots]
    it_one = [int(s.info[0]) for s in slots]
    t_b = timed(batched, max(1, args.steps))
    diff = max(float((s.u_out - u).abs().max()) for s, u in zip(slots, u_one))
    same_iters = all(int(s.info[0]) == k for s, k in zip(slots, it_one))
    n_pix = sum(wl.n_pix for wl in wls)
    evals = sum(int(s.info[2]) for s in slots)
    bytes_eval = sum(int(s.info[2]) * (B_PIX * wl.n_pix + B_NODE * wl.n_nodes) for s, wl in zip(slots, wls))
    peak, _ = peaks()
    return {"workload": "uneven_batch", "frames": n, "image_sides": sorted(set(int(w.ref.shape[0]) for w in wls)),
            "elements_px": sorted(set(int(w.name.split("_e")[1]) for w in wls)), "roi_pixels": n_pix,
            "batched_frames_per_s": n / t_b, "one_launch_per_frame_frames_per_s": n / t_one,
            "speedup": t_one / t_b, "batched_ms": 1000 * t_b, "one_by_one_ms": 1000 * t_one,
            "max_abs_diff_batched_vs_alone_px": diff, "same_iterations": same_iters,
            "objective_evaluations": evals,
            "roofline_frac_batched": (bytes_eval / 1e9 / t_b) / peak,
            "chunk_pixels_chosen": {str(c): shapes.count(c) for c in sorted(set(shapes))},
            "setup_s": {"assets": round(t_assets, 2), "autotune_and_layouts": round(t_tune, 2)}}


# ---------------------------------------------------------------------------
# local Gauss-Newton refinement chained after CG (the reference's published pipeline)
# ---------------------------------------------------------------------------

def run_local(args, dev, wl, dic):
    """3 local sweeps (lam 1e-3, max_step 0.2, omega 0.5) after each CG frame, as in the reference's
    PlateHole benchmark; timed on the workload's frames 1..5 from their CG solutions."""
    import torch

    import d2ic_gb300 as d2
    from dataclasses import replace as dc_replace
    loc = d2.DICMeshBased(wl.mesh, d2.LocalGaussNewtonSolver(device=dev),
                          dc_replace(wl.config, max_iters=3, save_history=True))
    loc.prepare(wl.ref, dic.state.assets)
    frames = list(range(1, min(6, len(wl.frames))))
    starts = []
    for k in frames:
        dic.set_initial_guess(None)
        starts.append(np.asarray(dic.run(wl.frames[k]).u_nodal))
    imgs = [torch.as_tensor(wl.frames[k], device=dev) for k in frames]
    loc.set_initial_guess(starts[0])
    loc.run(imgs[0])                                       # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = None
    for u0, img in zip(starts, imgs):
        loc.set_initial_guess(u0)
        r = loc.run(img)
        hist = r.history
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / len(frames)
    # discrepancy map of the last refined frame (MeshDICConfig.compute_discrepancy_map)
    from d2ic_gb300.pixel_maps import discrepancy_map_ref
    solver = dic.solver
    u_last = torch.as_tensor(np.asarray(r.u_nodal), device=dev)
    dmap, rms = discrepancy_map_ref(solver._layout, solver._desc_dev, imgs[-1], u_last)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(5):
        discrepancy_map_ref(solver._layout, solver._desc_dev, imgs[-1], u_last)
    torch.cuda.synchronize()
    return {"workload": wl.name, "sweeps_per_frame": 3, "ms_per_frame": 1000 * dt,
            "frames_per_s": 1.0 / dt, "last_history_rms_r_rms_step": np.asarray(hist).tolist(),
            "discrepancy_rms": rms, "discrepancy_ms": 1000 * (time.perf_counter() - t1) / 5}


def run_init_motion(args, dev, wl):
    """The first frame's initial motion: ZNCC integer search at the element centres and IDW onto the
    nodes (kernels timed alone with CUDA events), on the workload's frame 0, plus IDW at the largest
    mesh of the serving stream (4096^2 at 8 px: every grid node from every element centre)."""
    import torch

    from d2ic_gb300.dic_init_motion import project_centers_to_nodes_idw_device
    from d2ic_gb300.solver_translation_zncc import match_centers_device

    win, search = wl.init.win, wl.init.search
    centers = torch.as_tensor(np.asarray(wl.assets.element_centers_xy, dtype=np.float32), device=dev).reshape(-1, 2)
    ref = torch.as_tensor(wl.ref, device=dev)
    img = torch.as_tensor(wl.frames[0], device=dev)
    nodes = torch.as_tensor(np.asarray(wl.mesh.nodes_xy, dtype=np.float32), device=dev)

    def timed(fn, reps=10):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    u_c, sc = match_centers_device(centers, ref, img, win, search, dev)
    t_zncc = timed(lambda: match_centers_device(centers, ref, img, win, search, dev))
    t_idw = timed(lambda: project_centers_to_nodes_idw_device(nodes, centers, u_c, 2.0, dev))
    nc, nn = centers.shape[0], nodes.shape[0]
    npx, npa = win * win, (2 * search + 1) ** 2
    # FLOPs per offset: window sum (n adds), then per pixel centring (1), variance (2) and
    # cross-correlation (2): 6 n
    zflops = nc * npa * 6.0 * npx
    fp32_nominal = 152 * 128 * 2 * 2.07                     # GFLOP/s: 152 SMs x 128 lanes x FMA x 2.07 GHz
    # the serving stream's largest mesh: 4096^2 at 8 px, 513^2 nodes, 512^2 element centres
    g = torch.arange(0, 4097, 8, dtype=torch.float32, device=dev)
    big_nodes = torch.stack(torch.meshgrid(g, g, indexing="xy"), -1).reshape(-1, 2).contiguous()
    gc = torch.arange(4, 4096, 8, dtype=torch.float32, device=dev)
    big_centers = torch.stack(torch.meshgrid(gc, gc, indexing="xy"), -1).reshape(-1, 2).contiguous()
    big_disp = torch.randn(big_centers.shape, generator=torch.Generator(device=dev).manual_seed(4),
                           device=dev, dtype=torch.float32)
    t_big = timed(lambda: project_centers_to_nodes_idw_device(big_nodes, big_centers, big_disp, 2.0, dev), reps=2)
    pairs_big = big_nodes.shape[0] * big_centers.shape[0]
    return {"workload": wl.name, "centres": int(nc), "nodes": int(nn), "win": win, "search": search,
            "zncc_ms": t_zncc, "zncc_gflops": zflops / (t_zncc * 1e-3) / 1e9,
            "zncc_frac_of_nominal_fp32": zflops / (t_zncc * 1e-3) / 1e9 / fp32_nominal,
            "fp32_nominal_gflops": fp32_nominal, "idw_ms": t_idw,
            "idw_pairs_per_s": nc * nn / (t_idw * 1e-3),
            "idw_4096_e8": {"nodes": int(big_nodes.shape[0]), "centres": int(big_centers.shape[0]), "ms": t_big,
                            "pairs_per_s": pairs_big / (t_big * 1e-3)},
            "note": "zncc FLOPs per centre = offsets x 6 x window pixels; the FP32 peak is nominal "
                    "(no measured CUDA-core peak); both kernels run once per sequence (its first frame)"}


# ---------------------------------------------------------------------------
# implicit adjoint: noise propagation and finite differences
# ---------------------------------------------------------------------------

def run_adjoint(args, dev):
    """du*/dI2 for image-noise realisations (sigma 2) and its strain sensitivity, checked by FD."""
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300 import workloads
    from d2ic_gb300.adjoint import ImplicitAdjoint, newton_polish, strain_jvp
    from d2ic_gb300.mesh_assets import build_node_neighbor_tables

    wl = workloads.uniaxial_1024(device=dev)
    H, W = wl.ref.shape
    solver = d2.GlobalCGSolver(device=dev)
    dic = d2.DICMeshBased(wl.mesh, solver, wl.config)
    dic.prepare(wl.ref, wl.assets)
    img = torch.as_tensor(wl.frames[0], device=dev)
    res = dic.run(wl.frames[0])
    alpha = wl.config.reg_strength
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u = newton_polish(solver, dic.state, img, res.u_nodal, alpha, steps=2)
    slot = solver._ensure(dic.state)
    slot.load_image(img)
    adj = ImplicitAdjoint(slot, u, alpha)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    R = args.adjoint_realisations
    g = torch.Generator(device=dev).manual_seed(3000)
    noise = 2.0 * torch.randn((R, H, W), generator=g, device=dev, dtype=torch.float32)
    adj.jvp(noise, rtol=1e-6)                      # warm-up: work buffers sized for R right-hand sides
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    du = adj.jvp(noise, rtol=1e-6)
    torch.cuda.synchronize()
    t_jvp = time.perf_counter() - t0
    jvp_iters = adj.last_iters
    idx, deg = build_node_neighbor_tables(wl.mesh)
    dE = strain_jvp(u, du, np.asarray(wl.mesh.nodes_xy), idx, deg)
    used = torch.as_tensor(np.unique(np.asarray(wl.mesh.elements)), device=dev)
    u_std = du[:, used].std(dim=0)
    e_std = dE[:, used].std(dim=0)
    # VJP timing (one cotangent)
    gu = torch.zeros((1,) + tuple(u.shape), dtype=torch.float64, device=dev)
    gu[0, used, 0] = 1.0 / used.numel()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    adj.vjp(gu, rtol=1e-6)
    torch.cuda.synchronize()
    t_vjp = time.perf_counter() - t0
    # one Hessian matvec pass (J^T J v + springs) over all R right-hand sides with the assembled
    # node operator (the product the PCG runs), timed alone with CUDA events on its stream;
    # algorithmic bytes of the per-pixel form: 40 B per ROI pixel (image gradient 8 + node ids 16 +
    # shape functions 16) + 16 B per node per right-hand side; the kernel's own bytes: V read and Y
    # written once (16 B per node per right-hand side) + the operator (320 B per node)
    V = torch.randn((wl.n_nodes, 2, R), generator=g, device=dev, dtype=torch.float32)
    Y = torch.empty_like(V)
    st = torch.cuda.current_stream()
    adj.operator()

    def hv():
        adj.apply(V, Y)
    for _ in range(3):
        hv()
    reps = 20
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    clean = torch.ones(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    clean_sum = torch.empty((), dtype=torch.float32, device=dev)
    times = []
    for _ in range(reps):
        # V, Y and the operator start outside L2: write 256 MB, then read another 256 MB so that
        # L2 holds clean lines (the launch would otherwise also pay the write-back of the flush)
        flush.fill_(1.0)
        torch.sum(clean, dim=0, out=clean_sum)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        hv()
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    hv_ms = statistics.median(times)
    hv_bytes = 40 * wl.n_pix + 16 * R * wl.n_nodes
    hv_own = 16 * R * wl.n_nodes + (16 * 16 + 16 * 4) * wl.n_nodes
    peak, peak_src = peaks()
    hv_rate = hv_bytes / (hv_ms * 1e-3) / 1e9
    hv_own_rate = hv_own / (hv_ms * 1e-3) / 1e9
    # central finite differences of the exactly converged solution (Newton from u*)
    h = 1e-2
    D = args.adjoint_fd_dirs
    gd = torch.Generator(device=dev).manual_seed(3100)
    rels = []
    t0 = time.perf_counter()
    for k in range(D):
        d = torch.randn((1, H, W), generator=gd, device=dev, dtype=torch.float32)
        j = adj.jvp(d, rtol=1e-9)[0].to(torch.float64)
        up = newton_polish(solver, dic.state, img + h * d[0], u, alpha, steps=2).to(torch.float64)
        um = newton_polish(solver, dic.state, img - h * d[0], u, alpha, steps=2).to(torch.float64)
        fd = (up - um) / (2 * h)
        rels.append(float(torch.linalg.norm((fd - j)[used]) / torch.linalg.norm(j[used])))
    t_fd = time.perf_counter() - t0
    slot.load_image(img)
    return {"workload": "uniaxial_1024", "roi_pixels": wl.n_pix, "nodes": wl.n_nodes, "element_px": 12,
            "realisations": R, "noise_sigma": 2.0,
            "jvp_realisations_per_s": R / t_jvp, "jvp_s": t_jvp, "pcg_iterations": jvp_iters,
            "vjp_s": t_vjp, "setup_s": t_setup,
            "u_std_px_median": float(u_std.median()), "strain_std_median": [float(v) for v in e_std.median(dim=0).values],
            "fd_directions": D, "fd_h": h, "fd_rel_err_max": max(rels) if rels else None,
            "fd_rel_err_median": statistics.median(rels) if rels else None, "fd_s": t_fd,
            "hessian_matvec": {"kernel": "hop_apply (assembled node operator)", "rhs": R, "ms": hv_ms,
                               "algorithmic_bytes": hv_bytes, "achieved_GBps": hv_rate, "peak_GBps": peak,
                               "peak_source": peak_src, "frac": hv_rate / peak if peak else None,
                               "kernel_bytes": hv_own, "kernel_GBps": hv_own_rate,
                               "kernel_frac": hv_own_rate / peak if peak else None,
                               "l2": "flushed before each timed launch (256 MB write, then 256 MB read: clean lines)",
                               "note": "the Hessian is assembled once per linearisation point into per-node "
                                       "2x2 blocks, so a product reads V and the operator and writes Y; "
                                       "frac is against the per-pixel algorithmic bytes, kernel_frac "
                                       "against the kernel's own bytes"}}


# ---------------------------------------------------------------------------
# the engine at 4096^2 (frame data larger than L2: the HBM-bound case)
# ---------------------------------------------------------------------------

def run_engine_4096(args, dev):
    """The plate-hole sequence scaled to 4096^2 (11.8 M ROI pixels, 66,049 nodes): frames 1..n
    warm-started, engine launches timed with CUDA events on their stream, L2 flushed between
    steps; the same algorithmic bytes as the headline roofline."""
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300.sequence import SequenceRunner
    wl = make_workload("plate_hole_4096", 1 + args.frames_4096, 1, dev)
    solver = d2.GlobalCGSolver(device=dev)
    dic = d2.DICMeshBased(wl.mesh, solver, wl.config)
    dic.prepare(wl.ref, wl.assets)
    runner = SequenceRunner(solver, dic.state)
    frames_dev = [torch.from_numpy(f).to(dev) for f in wl.frames]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    runner.run(frames_dev, init_cfg=wl.init, propagation="previous")              # warm-up
    ms, evals = [], []
    for _ in range(max(1, min(args.steps, 3))):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        res = runner.run(frames_dev, init_cfg=wl.init, propagation="previous", time_engine=True)
        torch.cuda.synchronize()
        ms.extend(a.elapsed_time(b) for a, b in res.engine_events)
        evals.extend(res.info[:, 2].cpu().tolist())
    peak, peak_src = peaks()
    bpe = B_PIX * wl.n_pix + B_NODE * wl.n_nodes
    achieved = (sum(evals) * bpe / 1e9) / (sum(ms) / 1000.0)
    # admission cost of a new 4096^2 sequence: mesh from the mask (host), pixel assets as a device
    # recipe and the engine layout built on the device (second run timed; the first loads kernels)
    from d2ic_gb300.engine import FrameLayout
    from d2ic_gb300.pixel_assets import build_pixel_assets_device
    build_t = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mesh, assets = d2.mask_to_mesh_assets(wl.mask, 16)
        pd = build_pixel_assets_device(mesh, wl.ref, 1.0, assets.roi_mask)
        FrameLayout(pd, mesh.nodes_xy.shape[0], wl.ref, "cubic", dev)
        torch.cuda.synchronize()
        build_t.append(time.perf_counter() - t0)
    return {"workload": wl.name, "frames": len(frames_dev), "roi_pixels": wl.n_pix, "nodes": wl.n_nodes,
            "launch_ms_mean": statistics.mean(ms), "evals_per_launch": statistics.mean(evals),
            "us_per_eval": 1000.0 * sum(ms) / sum(evals), "bytes_per_eval": bpe, "achieved_GBps": achieved,
            "peak_GBps": peak, "peak_source": peak_src, "frac": achieved / peak,
            "sequence_setup_s": build_t[-1],
            "sequence_setup": "mask -> mesh (host) + pixel-asset recipe + engine layout on the device"}


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

def run_ours(args, ws, rank, local):
    import torch

    import d2ic_gb300 as d2
    from d2ic_gb300.sequence import SequenceRunner

    dev = torch.device("cuda", local)
    wl = make_workload(args.workload, args.frames, 1 + rank, dev)
    solver = d2.GlobalCGSolver(device=dev)
    dic = d2.DICMeshBased(wl.mesh, solver, wl.config)
    dic.prepare(wl.ref, wl.assets)
    runner = SequenceRunner(solver, dic.state)
    frames_dev = [torch.from_numpy(f).to(dev) for f in wl.frames]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    nF = len(frames_dev)

    def step(time_engine=False):
        return runner.run(frames_dev, init_cfg=wl.init, propagation="previous", time_engine=time_engine)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    engine_ms = []
    evals = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        res = step(time_engine=True)
        e1.record()
        barrier(ws)
        times.append(e0.elapsed_time(e1) / 1000.0)
        engine_ms.extend(a.elapsed_time(b) for a, b in res.engine_events)
        evals.extend(res.info[:, 2].cpu().tolist())
    clk = clocks.stop()
    t_step = max_over_ranks(statistics.median(times), ws)
    value = ws * nF / t_step
    iters = res.info[:, 0].cpu().tolist()

    # roofline of the persistent CG kernel
    peak, peak_src = peaks()
    bytes_per_eval = B_PIX * wl.n_pix + B_NODE * wl.n_nodes
    achieved = (sum(evals) * bytes_per_eval / 1e9) / (sum(engine_ms) / 1000.0)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "peak_source": peak_src, "kernel": "cg_engine<cubic>",
            "launch_ms_mean": statistics.mean(engine_ms), "evals_per_launch": statistics.mean(evals),
            "bytes_per_eval": bytes_per_eval}
    prof = os.path.join(ROOT, "profiles", "cg_engine_plate_hole_2048.txt")
    if os.path.exists(prof):
        for ln in open(prof):
            if ln.startswith("dram_bytes_per_eval:"):
                roof["traffic"] = float(ln.split(":")[1]) * statistics.mean(evals)

    out = {"metric": "frames/s", "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 (f64 CG reductions)", "data": "synthetic",
           "config": {"workload": wl.name, "frames": nF, "image": list(wl.ref.shape), "roi_pixels": wl.n_pix,
                      "nodes": wl.n_nodes, "element_px": 16, "tol": wl.config.tol, "reg": wl.config.reg_strength,
                      "max_iters": wl.config.max_iters, "l2": "flushed (256 MB write) between steps",
                      "parallelism": f"replicas x{ws}"},
           "cg_iterations_per_frame": statistics.mean(iters),
           "gpu_launches": nF * 4 + 2, "roofline": roof}
    if clk:
        out["clocks"] = clk

    # e2e through the public API with pinned host frames
    if not args.no_e2e:
        pinned = [torch.from_numpy(f).pin_memory() for f in wl.frames]
        init = d2.DICInitMotion(wl.init, d2.TranslationZNCCSolver(wl.init, device=dev))
        init.prepare(wl.ref, dic.state.assets)
        batch = d2.BatchMeshBased(wl.ref, dic.state.assets, dic, d2.BatchConfig(warm_start_from_previous=True))
        batch.before(pinned)

        def e2e_step():
            r0 = init.run(pinned[0])
            dic.set_initial_guess(r0.u_nodal)
            lat = []
            res = batch.sequence(pinned, latencies=lat)
            return res, lat

        for _ in range(max(1, args.warmup - 1)):
            e2e_step()
        et = []
        lats = []
        for _ in range(args.steps):
            barrier(ws)
            t0 = time.perf_counter()
            res_b, lat = e2e_step()
            barrier(ws)
            et.append(time.perf_counter() - t0)
            lats.extend(lat)
        te = max_over_ranks(statistics.median(et), ws)
        Nn = wl.n_nodes
        out["e2e"] = {"value": ws * nF / te, "unit": "frames/s",
                      "h2d_bytes_per_step": int(sum(f.nbytes for f in wl.frames)),
                      "d2h_bytes_per_step": int(nF * (Nn * 2 * 4 + Nn * 3 * 4 + wl.config.max_iters * 12 + 12)
                                                + Nn * 2 * 4),
                      "latency_ms_p50": 1000 * float(np.percentile(lats, 50)),
                      "latency_ms_p99": 1000 * float(np.percentile(lats, 99))}
        u_dev = res.u.cpu().numpy()
        u_api = np.stack([np.asarray(r.u_nodal) for r in res_b.results])
        out["e2e"]["max_abs_diff_vs_value_path_px"] = float(np.abs(u_dev - u_api).max())

    if not args.no_4096:
        out["engine_4096"] = run_engine_4096(args, dev)
    if not args.no_stream:
        out["serving_stream"] = run_serving_stream(args, dev)
    if not args.no_serve:
        if args.serve_mixed:                       # the reduced mixed stream (the serving stream supersedes it)
            out["serving"] = run_serving(args, dev)
        # the small-frame regime, where one frame alone cannot fill the GPU
        out["serving_small_frames"] = run_serving(args, dev, sides=(512,), n_seq=4 * args.serve_seqs,
                                                  label="small_frame_stream")
    if not args.no_local:
        out["local_refinement"] = run_local(args, dev, wl, dic)
        out["init_motion"] = run_init_motion(args, dev, wl)
    if not args.no_batch:
        out["batched"] = run_batched(args, dev)
    if not args.no_adjoint:
        out["adjoint"] = run_adjoint(args, dev)

    if not args.no_cpu and rank == 0:
        cb, sols = cpu_sequence_sample(wl, args.cpu_sample_frames, u_start=res.u[0].cpu().numpy())
        out["cpu_baseline"] = cb
        out["parity"] = parity_block(wl, res, sols)
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
