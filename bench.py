#!/usr/bin/env python
"""Benchmark: 65,536 uneven glyph-like paths rasterised to Matte8 masks (NonZero).

One step = one pass of the fill path over the whole batch (65,536 independent
Plotter::fill calls, each on its own canvas of side 16..256).

  value  Mpx/s with ops and masks resident in HBM: the prepared batch replays its
         CUDA graph (persistent kernel) K times, timed with CUDA events.
  e2e    the same metric through the C ABI call with host buffers
         (ft_fill_batch, FT_HOST): ops and rasters copied in, masks copied out,
         inside the timed region.
  cpu_baseline  the CPU oracle (a C++ restatement of footile's Plotter) on the
         host cores, one Plotter per path, on a bounded sample.

`--impl reference` times the CPU implementation alone (the reference is a Rust
crate and cannot be built here; its restatement is the timed CPU code).

Multi-GPU (torchrun): every rank renders its own 65,536-path batch (weak
scaling, no collective on the data path); value = all ranks' pixels / max time.
`--gpus N` (N > 1) outside torchrun starts the N ranks itself under
torch.distributed.run, so such a call never measures one GPU in their place.
"""
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
sys.path.insert(0, ROOT)

METRIC = "Mpx/s"
WORKLOAD = "glyphs_65536"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-paths", type=int, default=65536)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--per-path-sample", type=int, default=4096)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--no-tune", action="store_true", help="use the built-in plan instead of the autotuner")
    ap.add_argument("--tune-cache", default=None, help="autotuner cache file (looked up, then appended)")
    ap.add_argument("--composite-strokes", type=int, default=16384,
                    help="--only strokes / adjoint_composite: strokes on the 2048x2048 canvas")
    ap.add_argument("--composite-chunk", type=int, default=0,
                    help="--only adjoint_composite: strokes covered per chunk (0: sized to free memory)")
    ap.add_argument("--only", choices=["single", "scene", "strokes", "adjoint", "adjoint_strokes",
                                       "adjoint_composite"],
                    help="run one secondary workload alone (for profiling) and print its line")
    return ap.parse_args()


def _events_ms(stream, fn, reps):
    """Mean device time of fn() over `reps` calls, CUDA events on `stream`."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def extra_single(ctx, stream, dev, cpu=True):
    """One closed 64-segment path on 256x256 (Matte8 and Rgba8p), per call."""
    import ctypes
    import torch
    from footile_gb300 import _abi, workloads
    ops, w, h, clr = workloads.single_path_256()
    ops_d = torch.from_numpy(ops.view(np.uint8)).to(dev)
    m_d = torch.zeros((h, w), dtype=torch.uint8, device=dev)
    r_d = torch.zeros((h, w, 4), dtype=torch.uint8, device=dev)
    c = (ctypes.c_uint8 * 4)(*[int(v) for v in clr])
    L = ctx.L

    def fill(fmt, buf, stride):
        ctx.check(L.ft_fill(ctx.h, _abi.NONZERO, ctypes.c_void_p(ops_d.data_ptr()), len(ops), fmt, c,
                            ctypes.c_void_p(buf.data_ptr()), w, h, stride, _abi.DEVICE))
    for _ in range(5):
        fill(_abi.MATTE8, m_d, w)
    out = {"workload": "single_path_256 (64 mixed segments, 256x256, NonZero)",
           "matte8_us_per_call": 1e3 * _events_ms(stream, lambda: fill(_abi.MATTE8, m_d, w), 50),
           "rgba8p_us_per_call": 1e3 * _events_ms(stream, lambda: fill(_abi.RGBA8P, r_d, 4 * w), 50)}
    if cpu:
        import oracle
        r = np.zeros((h, w), np.uint8)
        t0 = time.perf_counter()
        for _ in range(50):
            oracle.fill(_abi.NONZERO, ops, r, _abi.MATTE8)
        out["cpu_oracle_us_per_call_1thread"] = (time.perf_counter() - t0) / 50 * 1e6
    return out


def extra_scene(ctx, stream, dev, cpu=True):
    """One 4096x4096 scene of 1,000 sub-paths x 100 segments: NonZero, EvenOdd, stroke."""
    import ctypes
    import torch
    from footile_gb300 import _abi, workloads
    from footile_gb300.path import PathOp, ops_array
    ops, w, h, clr = workloads.scene_4096()
    sops = np.concatenate([ops_array([PathOp.PenWidth(8.0)]), ops])
    ops_d = torch.from_numpy(ops.view(np.uint8)).to(dev)
    sops_d = torch.from_numpy(sops.view(np.uint8)).to(dev)
    m_d = torch.zeros((h, w), dtype=torch.uint8, device=dev)
    r_d = torch.zeros((h, w, 4), dtype=torch.uint8, device=dev)
    c = (ctypes.c_uint8 * 4)(*[int(v) for v in clr])
    L = ctx.L

    def fill(rule, fmt, buf, stride):
        ctx.check(L.ft_fill(ctx.h, rule, ctypes.c_void_p(ops_d.data_ptr()), len(ops), fmt, c,
                            ctypes.c_void_p(buf.data_ptr()), w, h, stride, _abi.DEVICE))

    def stroke():
        ctx.check(L.ft_stroke(ctx.h, ctypes.c_void_p(sops_d.data_ptr()), len(sops), _abi.MATTE8, c,
                              ctypes.c_void_p(m_d.data_ptr()), w, h, w, _abi.DEVICE))
    fill(_abi.NONZERO, _abi.MATTE8, m_d, w)
    out = {"workload": "scene_4096 (1,000 sub-paths x 100 segments; 65,535-vertex figure cap)",
           "nonzero_matte8_ms": _events_ms(stream, lambda: fill(_abi.NONZERO, _abi.MATTE8, m_d, w), 5),
           "evenodd_matte8_ms": _events_ms(stream, lambda: fill(_abi.EVENODD, _abi.MATTE8, m_d, w), 5),
           "nonzero_rgba8p_ms": _events_ms(stream, lambda: fill(_abi.NONZERO, _abi.RGBA8P, r_d, 4 * w), 5)}
    ctx.set_join(_abi.JOIN_ROUND, 0.0)
    stroke()
    out["stroke_w8_round_matte8_ms"] = _events_ms(stream, stroke, 3)
    ctx.set_join(_abi.JOIN_MITER, 4.0)
    # the un-capped extension: every sub-path kept (about 6 M vertices in one figure)
    ctx.set_figure_cap(8 << 20)
    fill(_abi.NONZERO, _abi.MATTE8, m_d, w)
    out["uncapped_nonzero_matte8_ms"] = _events_ms(stream, lambda: fill(_abi.NONZERO, _abi.MATTE8, m_d, w), 3)
    out["uncapped_coverage_fraction"] = float((m_d != 0).float().mean().item())
    # who builds the one large figure: the whole GPU (built-in from FT_GRID_BUILD_OPS ops)
    # or one CTA, capped and un-capped
    fb = {}
    for name, mode in (("grid", 2), ("one_cta", 1)):
        ctx.tune(fig_build=mode)
        for cap_name, cap in (("capped", 0), ("uncapped", 8 << 20)):
            ctx.set_figure_cap(cap)
            fill(_abi.NONZERO, _abi.MATTE8, m_d, w)
            fb[f"{name}_{cap_name}_nonzero_matte8_ms"] = _events_ms(
                stream, lambda: fill(_abi.NONZERO, _abi.MATTE8, m_d, w), 3)
        ctx.set_figure_cap(0)
        ctx.set_join(_abi.JOIN_ROUND, 0.0)
        stroke()
        fb[f"{name}_stroke_w8_round_matte8_ms"] = _events_ms(stream, stroke, 3)
        ctx.set_join(_abi.JOIN_MITER, 4.0)
    ctx.set_tuning(None)
    out["figure_build"] = fb
    ctx.set_figure_cap(0)
    # composite bytes: every Rgba8p pixel from the top row down is read and written
    out["rgba8p_composite_GBps"] = (w * h * 8) / (out["nonzero_rgba8p_ms"] * 1e-3) / 1e9
    # the compositing step alone (after the figure build and binning): by default the
    # call's coverage goes to a Matte8 mask and SrcOver streams canvas and mask through
    # shared memory by TMA; beside it the tile compositor (coverage and SrcOver fused),
    # TMA-staged and in place.  Roofline: 8 B per pixel (RGBA read and write; the mask
    # read adds 1 B) over the rows the call composites
    peak, peak_kind = measured_peak_hbm()
    comp = {}
    for name, stage in (("mask_then_tma_stream", 0), ("tile_tma_staged", 1), ("tile_in_place", 2)):
        ctx.tune(tile_stage=stage)
        fill(_abi.NONZERO, _abi.RGBA8P, r_d, 4 * w)
        t = []
        for _ in range(10):
            fill(_abi.NONZERO, _abi.RGBA8P, r_d, 4 * w)
            t.append(ctx.last_composite_ms())
        cms = float(np.median(t))
        comp[name] = {"ms": cms, "GBps": (w * h * 8) / (cms * 1e-3) / 1e9,
                      "frac_of_hbm": (w * h * 8) / (cms * 1e-3) / 1e9 / peak}
    ctx.set_tuning(None)
    out["rgba8p_tile_compositor"] = dict(comp, bytes=w * h * 8, peak=peak, peak_kind=peak_kind,
                                         tile=f"{ctx.tuning()['band_rows'] or 4} rows x "
                                              f"{ctx.tuning()['tile_w'] or 1024} px")
    # pix's Rgba8p -> SRgba8 step of footile's examples, on the device (HBM-bound):
    # the 4096x4096 raster, and an 8192x8192 one whose 512 MB of traffic is far above L2
    s_d = torch.empty_like(r_d)
    peak, _ = measured_peak_hbm()

    def kernel_ms(a, b, reps=10):  # device time of the conversion kernel (library events)
        ctx.convert(a, b)
        t = []
        for _ in range(reps):
            ctx.convert(a, b)
            t.append(ctx.last_ms())
        return float(np.median(t))
    out["srgba8_convert_4096_ms"] = kernel_ms(r_d, s_d)
    big = torch.randint(0, 256, (8192, 8192, 4), dtype=torch.uint8, device=dev)
    big_out = torch.empty_like(big)
    ms_conv = kernel_ms(big, big_out)
    out["srgba8_convert_8192_ms"] = ms_conv
    out["srgba8_convert_GBps"] = (8192 * 8192 * 8) / (ms_conv * 1e-3) / 1e9
    out["srgba8_convert_frac_of_measured_hbm"] = out["srgba8_convert_GBps"] / peak
    del big, big_out
    if cpu:
        import oracle
        m = np.zeros((h, w), np.uint8)
        t0 = time.perf_counter()
        oracle.fill(_abi.NONZERO, ops, m, _abi.MATTE8)
        out["cpu_oracle_nonzero_ms_1thread"] = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        oracle.stroke(sops, m, _abi.MATTE8, join=_abi.JOIN_ROUND, miter_limit=0.0)
        out["cpu_oracle_stroke_ms_1thread"] = (time.perf_counter() - t0) * 1e3
    return out


def extra_strokes(ctx, stream, dev, cpu=True, reps=2, n_paths=16384):
    """16,384 open cubic strokes (pen width 1..12, Miter(4)) composited in order onto
    one 2048x2048 Rgba8p canvas (ft_composite_batch)."""
    import torch
    from footile_gb300 import _abi, workloads
    from footile_gb300.plotter import composite_batch, pack_batch, pen_width_chain
    paths_ops, widths, clrs, side = workloads.strokes_16384(n_paths=n_paths)
    ops, paths, _ = pack_batch(paths_ops, [side] * len(paths_ops), _abi.RGBA8P, clrs)
    paths["s_width"], _ = pen_width_chain(ops, paths, 1.0)
    ops_d = torch.from_numpy(ops.view(np.uint8)).to(dev)
    ras_d = torch.zeros((side, side, 4), dtype=torch.uint8, device=dev)
    ctx.set_join(_abi.JOIN_MITER, 4.0)

    def run():
        composite_batch(ctx, ops_d, paths, _abi.RGBA8P, ras_d, stroke=True)
    run()
    t0 = time.perf_counter()
    dev_ms, comp_ms = [], []
    for _ in range(reps):
        run()
        dev_ms.append(ctx.last_ms())
        comp_ms.append(ctx.last_composite_ms())
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    # per-bbox algorithmic bytes of the ordered composite: every call reads and writes its
    # bounding box of RGBA (8 B/px) and its mask (1 B/px); the minimum is one canvas read
    # and write
    bbox_px = 0
    for o in paths_ops:
        pts = o["v"][1:, :6].reshape(-1, 2)
        lo = np.floor(pts.min(axis=0) - 6.0).clip(0, side)
        hi = np.ceil(pts.max(axis=0) + 6.0).clip(0, side)
        bbox_px += int(np.prod(hi - lo))
    peak, peak_kind = measured_peak_hbm()
    cms = float(np.median(comp_ms))
    out = {"workload": f"strokes_{n_paths} (8..64 cubics each, width 1..12, ordered SrcOver on 2048x2048 Rgba8p)",
           "ms_per_composite": ms, "paths_per_s": len(paths) / (ms * 1e-3),
           "canvas_Mpx_per_s": side * side / (ms * 1e-3) / 1e6,
           "device_ms": float(np.median(dev_ms)), "tile_compositor_ms": cms,
           "figure_build_and_bin_ms": float(np.median(dev_ms)) - cms,
           "compositor_roofline": {"bound": "hbm", "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                                   "bbox_bytes": 9 * bbox_px, "canvas_bytes": 2 * side * side * 4,
                                   "achieved_bbox": 9 * bbox_px / (cms * 1e-3) / 1e9 if cms else None,
                                   "frac_bbox": 9 * bbox_px / (cms * 1e-3) / 1e9 / peak if cms else None}}
    if cpu:
        # the reference composites every pixel from each call's top row down: time a few calls
        import oracle
        n = 8
        canvas = np.zeros((side, side, 4), np.uint8)
        t0 = time.perf_counter()
        oracle.composite(1, _abi.NONZERO, ops, paths[:n], _abi.RGBA8P, canvas)
        per = (time.perf_counter() - t0) / n
        out["cpu_oracle_ms_per_call_1thread"] = per * 1e3
        out["cpu_oracle_estimated_s_for_all_16384"] = per * len(paths)
    return out


def launch_ranks(args):
    """`--gpus N` with N > 1 outside torchrun: run this script as N ranks (one process
    per GPU) under torch.distributed.run on this node and return their exit status."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def config(args, world):
    full = args.n_paths == 65536
    return {"workload": WORKLOAD if full else f"glyphs_{args.n_paths}", "paths_per_gpu": args.n_paths,
            "canvas_side": "16..256 log-uniform",
            "segments": "4..400 log-uniform, 70% quad / 20% cubic / 10% line", "fill_rule": "NonZero",
            "format": "Matte8", "seed": "3 + rank", "parallelism": f"replicas x{world} (paths per rank)",
            "l2": "inputs larger than L2 (ops 185 MB + masks 780 MB per step)" if full else
                  "glyph batch smaller than the headline's (L2 share not stated)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
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
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled(key):
    """A per-launch figure of the rasteriser from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_raster_warp_glyphs_65536.txt")
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def profiled_traffic():
    """DRAM bytes per launch of the rasteriser (dram__bytes_read.sum + write.sum)."""
    return profiled("traffic_bytes_per_launch")


def accumulation(kernel_ms):
    wf = profiled("shared_atomic_wavefronts_per_launch")
    if wf is None:
        return None
    return {"bound": "shared-memory atomics", "wavefronts_per_launch": wf,
            "warp_instructions_per_launch": profiled("shared_atomic_warp_insts_per_launch"),
            "achieved": wf / (kernel_ms * 1e-3) / 1e9, "unit": "G atomic wavefronts/s",
            "utilisation_pct_of_peak": profiled("shared_atomic_pipe_pct_of_peak"),
            "source": "profiles/k_raster_warp_glyphs_65536.txt"}


def cpu_baseline(ops, paths, nbytes, seconds, threads, gpu_masks=None):
    """Time the oracle on a bounded sample of the workload (all host threads).  With
    `gpu_masks` (the timed batch's rasters, copied to the host), the oracle's masks of
    every path (the timed sample, then the rest outside the timing) are compared with
    them byte for byte: returns (baseline, parity)."""
    import oracle
    from footile_gb300 import _abi
    px = paths["width"].astype(np.int64) * paths["height"]
    probe = min(512, len(paths))
    r = np.zeros(nbytes, np.uint8)
    t0 = time.perf_counter()
    oracle.fill_batch(0, _abi.NONZERO, ops, paths[:probe], _abi.MATTE8, r, n_threads=threads)
    dt = time.perf_counter() - t0
    rate = probe / max(dt, 1e-6)
    n = int(min(len(paths), max(probe, rate * seconds)))
    t0 = time.perf_counter()
    oracle.fill_batch(0, _abi.NONZERO, ops, paths[:n], _abi.MATTE8, r, n_threads=threads)
    dt = time.perf_counter() - t0
    base = {"value": float(px[:n].sum() / dt / 1e6), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"first {n} of {len(paths)} paths ({int(px[:n].sum())} px), one Plotter per path",
            "paths_per_s": n / dt, "seconds": dt}
    if gpu_masks is None:
        return base, None
    if n < len(paths):
        oracle.fill_batch(0, _abi.NONZERO, ops, paths[n:], _abi.MATTE8, r, n_threads=threads)
    bad = np.flatnonzero(r != gpu_masks)
    bad_paths = np.unique(np.searchsorted(paths["raster_offset"].astype(np.int64), bad, side="right") - 1)
    parity = {"paths_checked": int(len(paths)), "mismatching_paths": int(len(bad_paths)),
              "bytes_compared": int(nbytes), "mismatching_bytes": int(len(bad)), "bit_exact": len(bad) == 0,
              "against": "oracle masks of every path of the timed batch (initial rasters zero on both sides)"}
    return base, parity


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from footile_gb300 import workloads
    ops, paths, nbytes = workloads.glyphs(args.n_paths, seed=3)
    threads = os.cpu_count() or 1
    px = paths["width"].astype(np.int64) * paths["height"]
    import oracle
    from footile_gb300 import _abi
    # each step: a bounded sample of the workload sized so the run stays within minutes
    r = np.zeros(nbytes, np.uint8)
    probe = min(256, len(paths))
    t0 = time.perf_counter()
    oracle.fill_batch(0, _abi.NONZERO, ops, paths[:probe], _abi.MATTE8, r, n_threads=threads)
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    budget = 120.0 / max(args.steps + args.warmup, 1)
    n = int(min(len(paths), max(probe, rate * budget)))
    sample = paths[:n]
    for _ in range(args.warmup):
        oracle.fill_batch(0, _abi.NONZERO, ops, sample, _abi.MATTE8, r, n_threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.fill_batch(0, _abi.NONZERO, ops, sample, _abi.MATTE8, r, n_threads=threads)
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    val = float(px[:n].sum() / dt / 1e6)
    desc = f"first {n} of {len(paths)} paths per step ({int(px[:n].sum())} px)"
    out = {"metric": METRIC, "value": val, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int32 (16.16 fixed) + f32", "data": "synthetic",
           "config": config(args, world),
           "cpu_baseline": {"value": val, "unit": METRIC, "cores": threads, "kind": "port", "sample": desc},
           "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "footile is a Rust crate; no cargo/rustc in this image, so the timed CPU code is its C++ "
                   "restatement (oracle/footile_oracle.cpp), one Plotter per path on all host threads"}
    print(json.dumps(out), flush=True)


def extra_adjoint(ctx, stream, dev, cpu=True, reps=10, check_paths=32, fd_paths=2):
    """Coverage adjoint on 1,024 closed 32-cubic paths (128x128 f32 coverage each):
    forward and backward device time, and the gradient's error against the FP64 oracle
    and against central differences (h = 1e-2 px) of the FP64 coverage."""
    import torch
    from footile_gb300 import _abi, workloads
    from footile_gb300.adjoint import Adjoint
    ops, paths, cov_bytes, target = workloads.cubics_1024_coverage()
    n_px = cov_bytes // 4
    ops_d = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
    tgt_d = torch.from_numpy(target).to(dev)
    cov_d = torch.empty(n_px, dtype=torch.float32, device=dev)
    gops_d = torch.empty((len(ops), 6), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # larger than L2
    adj = Adjoint(ctx)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    fwd, bwd, fwd_k, bwd_k = [], [], [], []
    for it in range(reps + 3):
        flush.zero_()
        e[0].record(stream)
        adj.forward(_abi.NONZERO, ops_d, paths, cov_d)
        e[1].record(stream)
        fk = ctx.last_ms()
        g_cov = 2.0 * (cov_d - tgt_d)  # dLoss/dcov of sum((cov - target)^2), outside both timings
        flush.zero_()
        e[2].record(stream)
        adj.backward(g_cov, gops_d)
        e[3].record(stream)
        bk = ctx.last_ms()
        torch.cuda.synchronize()
        if it >= 3:
            fwd.append(e[0].elapsed_time(e[1]))
            bwd.append(e[2].elapsed_time(e[3]))
            fwd_k.append(fk)
            bwd_k.append(bk)
    st = adj.status()
    out = {"workload": "cubics_1024 coverage adjoint (1,024 closed paths x 32 cubics, 128x128 f32, L2 loss)",
           "fwd_ms": float(np.median(fwd)), "bwd_ms": float(np.median(bwd)),
           "fwd_kernel_ms": float(np.median(fwd_k)), "bwd_kernel_ms": float(np.median(bwd_k)),
           "bwd_over_fwd": float(np.median(bwd) / np.median(fwd)), "paths_status_ok": int((st == 0).sum()),
           "l2_flushed_between_calls": True}
    if cpu:
        import oracle
        cov = cov_d.cpu().numpy()
        g = gops_d.cpu().numpy().astype(np.float64)
        gc = (2.0 * (cov.astype(np.float64) - target)).astype(np.float32).astype(np.float64)
        num, den = 0.0, 0.0
        t0 = time.perf_counter()
        for p in paths[:check_paths]:
            b, n = int(p["op_begin"]), int(p["n_ops"])
            o = ops[b:b + n]
            c64, area, _ = oracle.adj_forward(_abi.NONZERO, o, 128, 128)
            off = int(p["raster_offset"]) // 4
            r = oracle.adj_backward(_abi.NONZERO, o, 128, 128, area, gc[off:off + 128 * 128].reshape(128, 128))
            num = max(num, float(np.abs(g[b:b + n] - r).max()))
            den = max(den, float(np.abs(r).max()))
        out["cpu_fp64_oracle_ms_per_path_fwd_bwd"] = (time.perf_counter() - t0) / check_paths * 1e3
        out["max_rel_err_vs_fp64"] = num / den
        out["rel_err_definition"] = "max|g - g64| / max|g64| over the op floats of the first %d paths" % check_paths
        # central differences of the FP64 loss (subdivision tree held), all 198 floats of a path
        fd_num, fd_den = 0.0, 0.0
        for p in paths[:fd_paths]:
            b, n = int(p["op_begin"]), int(p["n_ops"])
            o = ops[b:b + n]
            off = int(p["raster_offset"]) // 4
            tg = target[off:off + 128 * 128].reshape(128, 128).astype(np.float64)
            c64, area, _ = oracle.adj_forward(_abi.NONZERO, o, 128, 128)
            r = oracle.adj_backward(_abi.NONZERO, o, 128, 128, area, 2 * (c64 - tg))
            base = np.array([x["v"] for x in o], dtype=np.float64)
            fd = np.zeros_like(base)
            for i in range(n):
                for k in range(6):
                    if o[i]["kind"] in (_abi.OP_CLOSE, _abi.OP_PEN_WIDTH) or (o[i]["kind"] != _abi.OP_CUBIC and k >= 2):
                        continue
                    vp, vm = base.copy(), base.copy()
                    vp[i, k] += 1e-2
                    vm[i, k] -= 1e-2
                    lp = ((oracle.adj_forward(_abi.NONZERO, o, 128, 128, val=vp)[0] - tg) ** 2).sum()
                    lm = ((oracle.adj_forward(_abi.NONZERO, o, 128, 128, val=vm)[0] - tg) ** 2).sum()
                    fd[i, k] = (lp - lm) / 2e-2
            fd_num = max(fd_num, float(np.abs(g[b:b + n] - fd).max()))
            fd_den = max(fd_den, float(np.abs(fd).max()))
        out["max_rel_err_vs_central_fd_h1e-2"] = fd_num / fd_den
        out["fd_paths"] = fd_paths
    adj.close()
    return out


def extra_adjoint_strokes(ctx, stream, dev, cpu=True, reps=5, n_paths=1024, side=256, check_paths=8):
    """Stroke coverage adjoint on 1,024 open strokes shaped like the ordered-composite
    workload (8..64 cubics, PenWidth 1..12, Miter(4)), each on its own 256x256 f32
    coverage plane: forward / backward device time and the error of the op-float and
    pen-width gradients against the FP64 oracle (and central differences, h = 1e-2)."""
    import torch
    from footile_gb300 import _abi, workloads
    from footile_gb300.adjoint import Adjoint, pack_coverage
    paths_ops, _, _, _ = workloads.strokes_16384(n_paths=n_paths, side=side)
    ops, paths, cov_bytes = pack_coverage(paths_ops, [side] * n_paths)
    target = np.random.default_rng(5).random(cov_bytes // 4, dtype=np.float32)
    ops_d = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
    tgt_d = torch.from_numpy(target).to(dev)
    cov_d = torch.empty(cov_bytes // 4, dtype=torch.float32, device=dev)
    gops_d = torch.empty((len(ops), 6), dtype=torch.float32, device=dev)
    gw_d = torch.empty(n_paths, dtype=torch.float32, device=dev)
    ctx.set_join(_abi.JOIN_MITER, 4.0)
    adj = Adjoint(ctx)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    fwd, bwd = [], []
    for it in range(reps + 2):
        e[0].record(stream)
        adj.forward(_abi.NONZERO, ops_d, paths, cov_d, stroke=True)
        e[1].record(stream)
        g_cov = 2.0 * (cov_d - tgt_d)
        e[2].record(stream)
        adj.backward(g_cov, gops_d, gw_d)
        e[3].record(stream)
        torch.cuda.synchronize()
        if it >= 2:
            fwd.append(e[0].elapsed_time(e[1]))
            bwd.append(e[2].elapsed_time(e[3]))
    st = adj.status()
    out = {"workload": "strokes adjoint (1,024 open strokes, 8..64 cubics, width 1..12, Miter(4), 256x256 f32 each)",
           "fwd_ms": float(np.median(fwd)), "bwd_ms": float(np.median(bwd)),
           "bwd_over_fwd": float(np.median(bwd) / np.median(fwd)), "paths_status_ok": int((st == 0).sum())}
    if cpu:
        import oracle
        cov = cov_d.cpu().numpy()
        g = gops_d.cpu().numpy().astype(np.float64)
        gw = gw_d.cpu().numpy().astype(np.float64)
        gc = (2.0 * (cov.astype(np.float64) - target)).astype(np.float32).astype(np.float64)
        num, den = 0.0, 0.0
        for i, p in enumerate(paths[:check_paths]):
            b, n = int(p["op_begin"]), int(p["n_ops"])
            o = ops[b:b + n]
            c64, area, _ = oracle.adj_stroke_forward(o, side, side)
            off = int(p["raster_offset"]) // 4
            r, rw = oracle.adj_stroke_backward(o, side, side, area, gc[off:off + side * side].reshape(side, side))
            num = max(num, float(np.abs(g[b:b + n] - r).max()), abs(gw[i] - rw))
            den = max(den, float(np.abs(r).max()), abs(rw))
        out["max_rel_err_vs_fp64"] = num / den
        out["paths_checked"] = check_paths
        # central differences (h = 1e-2) of the FP64 loss for the PenWidth op of path 0
        p = paths[0]
        b, n = int(p["op_begin"]), int(p["n_ops"])
        o = ops[b:b + n]
        off = int(p["raster_offset"]) // 4
        tg = target[off:off + side * side].reshape(side, side).astype(np.float64)
        base = np.array([x["v"] for x in o], dtype=np.float64)
        lo = lambda v: ((oracle.adj_stroke_forward(o, side, side, val=v)[0] - tg) ** 2).sum()
        vp, vm = base.copy(), base.copy()
        vp[0, 0] += 1e-2
        vm[0, 0] -= 1e-2
        fd_w = (lo(vp) - lo(vm)) / 2e-2
        out["pen_width_grad_path0"] = float(g[b, 0])
        out["pen_width_central_fd_h1e-2_path0"] = float(fd_w)
    adj.close()
    return out


def extra_adjoint_composite(ctx, stream, dev, cpu=True, n_paths=16384, side=2048, reps=2, chunk=0):
    """Differentiable ordered composite at full size: 16,384 open strokes of 8..64 cubics,
    width 1..12, Miter(4), colours with alpha 64..255, SrcOver'd in order on one 2048x2048
    canvas, L2 loss against a seeded RGBA target; gradients of the control points and pen
    widths (ft_stroke_composite_forward / _backward: coverage in chunks sized to the
    free memory, recomputed chunk by chunk in the backward).  The FP64 chain checks the
    first 24 strokes on the same canvas."""
    import torch
    from footile_gb300 import _abi, workloads
    from footile_gb300.adjoint import StrokeComposite, pack_coverage, stroke_composite_grads
    torch.cuda.empty_cache()  # the chunk size follows the free device memory
    paths_ops, _, clrs, _ = workloads.strokes_16384(n_paths=n_paths, side=side)
    ops, paths, _ = pack_coverage(paths_ops, [side] * n_paths)
    clr = clrs.astype(np.float32) / 255.0
    target = np.random.default_rng(7).random((side * side, 4), dtype=np.float32)
    ops_d = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
    clr_d = torch.from_numpy(clr).to(dev)
    tgt_d = torch.from_numpy(target).to(dev)
    ctx.set_join(_abi.JOIN_MITER, 4.0)
    comp = StrokeComposite(ctx)
    stroke_composite_grads(ctx, ops_d, paths, clr_d, side, side, tgt_d, comp, chunk)  # warm-up (allocations)
    runs = []
    t0 = time.perf_counter()
    for _ in range(reps):
        loss, out, g_ops, g_w, ms = stroke_composite_grads(ctx, ops_d, paths, clr_d, side, side, tgt_d, comp, chunk)
        runs.append(ms)
    wall = (time.perf_counter() - t0) / reps * 1e3
    st = comp.status()
    res = {"workload": f"strokes composite adjoint ({n_paths:,} strokes, 8..64 cubics, width 1..12, Miter(4), "
                       f"ordered SrcOver on one {side}x{side} canvas, L2 loss vs RGBA target)",
           "fwd_ms": float(np.median([r["fwd_ms"] for r in runs])),
           "bwd_ms": float(np.median([r["bwd_ms"] for r in runs])), "wall_ms_per_fwd_bwd": wall,
           "chunk": runs[-1]["chunk"], "n_chunks": -(-n_paths // runs[-1]["chunk"]),
           "paths_status_ok": int((st == _abi.OK).sum()), "loss": float(loss),
           "grad_finite": bool(torch.isfinite(g_ops).all().item() and torch.isfinite(g_w).all().item())}
    res["bwd_over_fwd"] = res["bwd_ms"] / res["fwd_ms"]
    comp.close()
    if cpu:
        # FP64 chain on the first 24 strokes (their own composite on the same canvas)
        import oracle
        k = 24
        o2, p2, _ = pack_coverage(paths_ops[:k], [side] * k)
        o2_d = torch.from_numpy(o2.view(np.uint8).copy()).to(dev)
        l2, out2, g2, gw2, _ = stroke_composite_grads(ctx, o2_d, p2, clr_d[:k].contiguous(), side, side, tgt_d)
        t1 = time.perf_counter()
        l64, C64, g64, gw64 = oracle.adj_stroke_composite(o2, p2, clr[:k].astype(np.float64), side, side,
                                                          target.astype(np.float64))
        res["cpu_fp64_chain_s_for_24"] = time.perf_counter() - t1
        scale = max(np.abs(g64).max(), np.abs(gw64).max())
        res["max_rel_err_vs_fp64_24_strokes"] = float(max(np.abs(g2.cpu().numpy() - g64).max(),
                                                          np.abs(gw2.cpu().numpy() - gw64).max()) / scale)
        res["max_abs_canvas_err_24_strokes"] = float(np.abs(out2.cpu().numpy() - C64).max())
    return res


def run_only(args):
    import torch
    from footile_gb300._lib import Context
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx = Context(0)
    ctx.set_stream(stream.cuda_stream)
    fn = {"single": extra_single, "scene": extra_scene, "strokes": extra_strokes, "adjoint": extra_adjoint,
          "adjoint_strokes": extra_adjoint_strokes, "adjoint_composite": extra_adjoint_composite}[args.only]
    kw = {}
    if args.only == "adjoint_composite":
        kw = {"n_paths": args.composite_strokes, "chunk": args.composite_chunk}
    elif args.only == "strokes":
        kw = {"n_paths": args.composite_strokes}
    print(json.dumps(fn(ctx, stream, dev, cpu=not args.no_cpu, **kw)), flush=True)


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but {world} rank(s) were started")
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from footile_gb300 import _abi, workloads
    from footile_gb300._lib import Context
    from footile_gb300.plotter import PreparedBatch

    ops, paths, nbytes = workloads.glyphs(args.n_paths, seed=3 + rank)
    px_total = int((paths["width"].astype(np.int64) * paths["height"]).sum())
    n_ops = len(ops)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)  # a capturable stream for the batch's CUDA graph
    torch.cuda.set_stream(stream)
    ctx = Context(local)
    ctx.set_stream(stream.cuda_stream)
    ops_d = torch.from_numpy(ops.view(np.uint8)).to(dev)
    ras_d = torch.zeros(nbytes, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()

    # ---- plan: the built-in one, then the autotuner's choice (both outside the timed region)
    def launch_ms(b, reps=5):
        b.launch(ops_d, ras_d)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(reps):
            b.launch(ops_d, ras_d)
        a1.record(stream)
        torch.cuda.synchronize()
        return a0.elapsed_time(a1) / reps
    tune_info = {"autotuned": False}
    if not args.no_tune:
        b0 = PreparedBatch(ctx, paths, _abi.MATTE8)
        tune_info["default_plan_ms"] = launch_ms(b0)
        tune_info["default_plan"] = ctx.tuning()
        b0.close()
        t0 = time.perf_counter()
        chosen, tms = ctx.autotune(ops_d, paths, _abi.MATTE8, ras_d, cache_path=args.tune_cache)
        tune_info.update({"autotuned": True, "chosen_plan": chosen, "chosen_plan_ms_while_tuning": tms,
                          "tuning_s": time.perf_counter() - t0})
    batch = PreparedBatch(ctx, paths, _abi.MATTE8)

    from footile_gb300 import replicas

    def barrier():
        replicas.barrier()

    for _ in range(args.warmup):
        batch.launch(ops_d, ras_d)
    st = batch.status()
    assert (st == 0).all(), f"path status errors: {np.unique(st)}"

    # ---- device-resident throughput (value)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launch_count()
    e0.record(stream)
    for _ in range(args.steps):
        batch.launch(ops_d, ras_d)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = ctx.launch_count() - launches0
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    # the timed graph's masks, for the parity check against the oracle
    gpu_masks = ras_d.cpu().numpy() if (rank == 0 and world == 1 and not args.no_cpu) else None
    # per-launch device time of the graph (memsets + rasteriser), library events
    kms = []
    for _ in range(args.steps):
        batch.launch(ops_d, ras_d)
        kms.append(ctx.last_ms())
    clk = clocks.stop()
    # every rank renders its own batch: job pixels over the slowest rank's time
    ms_max = replicas.reduce_max(ms, dev)
    job_px = replicas.reduce_sum(px_total, dev)
    value = job_px / (ms_max * 1e-3) / 1e6

    # ---- end to end through the C ABI with host buffers (e2e)
    from footile_gb300.plotter import fill_batch
    ops_h = torch.from_numpy(ops.view(np.uint8)).pin_memory()
    ras_h = torch.zeros(nbytes, dtype=torch.uint8).pin_memory()
    ops_np = ops_h.numpy().view(_abi.OP_DTYPE)
    ras_np = ras_h.numpy()
    ctx2 = Context(local)
    ctx2.set_tuning(ctx.tuning())
    fill_batch(ctx2, ops_np, paths, _abi.MATTE8, ras_np)  # warm (allocations)
    barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 5))
    for _ in range(e2e_steps):
        fill_batch(ctx2, ops_np, paths, _abi.MATTE8, ras_np)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    barrier()
    e2e_s = replicas.reduce_max(e2e_s, dev)
    e2e_val = job_px / e2e_s / 1e6
    # masks of the e2e path must equal the device path's
    same = bool(np.array_equal(ras_np, ras_d.cpu().numpy()))
    # The pinned Matte8 rasters above are written in place by the kernels over the host
    # link; the copy pipeline (rasters copied in, drawn, copied out in two overlapped
    # chunks) is timed beside it with the mapping switched off.
    mapped = ctx2.tuning()["host_mapped"] == 0
    ctx2.tune(host_mapped=1)  # ops and rasters copied in, rasters copied out
    fill_batch(ctx2, ops_np, paths, _abi.MATTE8, ras_np)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        fill_batch(ctx2, ops_np, paths, _abi.MATTE8, ras_np)
    e2e_copy_s = replicas.reduce_max((time.perf_counter() - t0) / e2e_steps, dev)
    same = same and bool(np.array_equal(ras_np, ras_d.cpu().numpy()))

    # ---- one launch per path (ft_fill, device mode), on a sample
    per_path = None
    if rank == 0 and args.per_path_sample > 0:
        import ctypes
        n = min(args.per_path_sample, len(paths))
        sub_px = int((paths["width"][:n].astype(np.int64) * paths["height"][:n]).sum())
        L = ctx.L
        base_o, base_r = ops_d.data_ptr(), ras_d.data_ptr()
        clr = (ctypes.c_uint8 * 4)(0, 0, 0, 0)

        def one(i):
            d = paths[i]
            rc = L.ft_fill(ctx.h, _abi.NONZERO, ctypes.c_void_p(base_o + 32 * int(d["op_begin"])), int(d["n_ops"]),
                           _abi.MATTE8, clr, ctypes.c_void_p(base_r + int(d["raster_offset"])), int(d["width"]),
                           int(d["height"]), int(d["stride"]), _abi.DEVICE)
            ctx.check(rc)
        for i in range(min(64, n)):
            one(i)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(n):
            one(i)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        per_path = {"paths_per_s": n / dt, "mpx_per_s": sub_px / dt / 1e6, "sample_paths": n,
                    "launches_per_path": 1}

    # ---- the other configurations, on rank 0 (device time, CUDA events)
    extras = None
    ctx.set_tuning(None)  # the other workloads use the built-in plans
    if rank == 0 and not args.no_extras:
        extras = {}
        for name, fn in (("single_path_256", extra_single), ("scene_4096", extra_scene),
                         ("strokes_16384", extra_strokes), ("adjoint_cubics_1024", extra_adjoint),
                         ("adjoint_strokes_1024", extra_adjoint_strokes),
                         ("adjoint_composite_16384", extra_adjoint_composite)):
            try:
                extras[name] = fn(ctx, stream, dev, cpu=(world == 1 and not args.no_cpu))
            except Exception as e:  # report, never hide, a failing secondary workload
                extras[name] = {"error": repr(e)}

    # ---- CPU baseline (rank 0, N=1 only)
    cpu, parity = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, parity = cpu_baseline(ops, paths, nbytes, args.cpu_seconds, os.cpu_count() or 1, gpu_masks)

    if rank != 0:
        return
    peak, peak_kind = measured_peak_hbm()
    alg_bytes = px_total + 32 * n_ops + 40 * len(paths)
    kmean = float(np.mean(kms)) if kms else ms
    achieved = alg_bytes / (kmean * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32 (16.16 fixed) + f32", "data": "synthetic",
        "config": config(args, world),
        "paths_per_s": len(paths) * world / (ms_max * 1e-3),
        "e2e": {"value": e2e_val, "unit": METRIC,
                "h2d_bytes_per_step": int(32 * n_ops + 40 * len(paths) + (0 if mapped else nbytes)),
                "d2h_bytes_per_step": int(nbytes), "ms_per_step": e2e_s * 1e3, "masks_equal_device_path": same,
                "rasters": ("pinned host memory written in place by the kernels over the host link (every "
                            "raster row a figure reaches; the rest keep the host's bytes)") if mapped else
                           "copied in, drawn and copied out in two overlapped chunks",
                "copy_pipeline": {"value": job_px / e2e_copy_s / 1e6, "ms_per_step": e2e_copy_s * 1e3,
                                  "h2d_bytes_per_step": int(32 * n_ops + nbytes + 40 * len(paths)),
                                  "d2h_bytes_per_step": int(nbytes)}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profiled_traffic() if args.n_paths == 65536 else None, "peak_kind": peak_kind,
                     "kernel": "ftk::k_raster_warp<false> + ftk::k_raster<false> (graph: 2 memsets, warp rasteriser, CTA rasteriser)", "kernel_ms": kmean,
                     "algorithmic_bytes_per_launch": int(alg_bytes)},
        # the cell accumulation's bound: shared-memory atomics (data-path wavefronts of one
        # launch from the ncu summary, over this run's kernel time; the atomic data path's
        # utilisation as ncu measured it)
        "accumulation": accumulation(kmean),
        "cpu_baseline": cpu,
        "parity": parity,
        "modes": {"batched_paths_per_s": len(paths) / (ms_max * 1e-3), "per_path_launch": per_path,
                  "batched_over_per_path": (len(paths) / (ms_max * 1e-3) / per_path["paths_per_s"]) if per_path else None},
        "clocks": clk,
        "gpu_launches": int(launches),
        "plan": tune_info,
        "workloads": extras,
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args))
    if args.impl == "reference":
        run_reference(args)
    elif args.only:
        run_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
