"""Benchmark: field points*modes/s of the GB300 field evaluator.

One step = one evaluation of the whole workload grid against the sample's plane waves,
inputs already resident in HBM (``value``); ``e2e`` times the same work through the
host-buffer C-ABI calls (wave upload from pinned host memory + evaluation + read-back).

Work unit (points*modes): sum over evaluated points of the number of plane waves in the
point's region (waves_end[l] - waves_begin[l], cpuEvaluator.cpp:34-53) -- identical for
the plain and the separable (GEMM) form.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Multi-GPU (torchrun): every rank evaluates its own copy of the workload (weak scaling,
no data exchange); value = all ranks' units / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "field points*modes/s"
UNIT = "points*modes/s"

# The sphere workload at [20, 64, 64] with 20 x 20 harmonics: 128 x 128 x 64 grid over
# x, y in [-32, 32] and z over the sample +-10 units.
CFG1 = dict(name="spheres[20,64,64] coef20x20 grid128x128x64", M0=20, M1=20, Z=20, size=(64.0, 64.0, 20.0),
            Nx=128, Ny=128, Nz=64, x0=-32.0, y0=-32.0, z0=-20.0, x1=32.0, y1=32.0, z1=20.0)


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def region_counts(begin, end, zl, rule, zs):
    """Number of waves seen by each z value (reference region rule)."""
    zf = np.asarray(zl, np.float32).astype(np.float64)
    thr = zf - 0.001 if rule == 0 else zf
    out = []
    for z in np.asarray(zs, np.float32).astype(np.float64):
        l = 0
        for li in range(len(thr)):
            if z >= thr[li]:
                l = li + 1
        out.append(int(end[l] - begin[l]))
    return np.array(out, dtype=np.int64)


def grid_axis(s, d, n):
    return (np.float32(s) + np.float32(d) * np.arange(n, dtype=np.float32)).astype(np.float32)


def build_workload(cfg, seed=0):
    from scwatter_gb300 import synthetic
    fs = synthetic.make_factored(cfg["M0"], cfg["M1"], cfg["Z"], cfg["size"], seed=seed)
    Pi, zs, Pr, Pt = synthetic.to_cw_arrays(fs)
    dx = np.float32((cfg["x1"] - cfg["x0"]) / (cfg["Nx"] - 1))
    dy = np.float32((cfg["y1"] - cfg["y0"]) / (cfg["Ny"] - 1))
    dz = np.float32((cfg["z1"] - cfg["z0"]) / (cfg["Nz"] - 1))
    return fs, (Pi, zs, Pr, Pt), (dx, dy, dz)


def unpack_arrays(Pi, zs, Pr, Pt):
    parts = [Pi]
    begin, end = [0], []
    total = len(Pi)
    for l in range(len(zs)):
        total += len(Pr[l])
        end.append(total)
        begin.append(total)
        total += len(Pt[l])
        parts += [Pr[l], Pt[l]]
    end.append(total)
    return np.concatenate(parts), np.array(begin), np.array(end), np.array(zs)


def cpu_reference_rate(W32, begin, end, zl, cfg, d, target_s=10.0, threads=None):
    """Reference FP32 CPU evaluator (cpu_cw_evaluate_xy restated) on a bounded sample: rows of
    the interior xy plane nearest the sample centre, all host threads."""
    from oracle import oracle_lib as ol
    threads = threads or ol.default_threads()
    dx, dy, dz = d
    zs = grid_axis(cfg["z0"], dz, cfg["Nz"])
    counts = region_counts(begin, end, zl, 1, zs)
    iz = int(np.argmax(counts))
    z = float(zs[iz])
    N = cfg["Nx"]
    # calibrate with one row per thread
    rows = threads
    t0 = time.perf_counter()
    ol.cpu_eval_plane_f32(ol.AXIS_XY, W32, begin, end, zl, cfg["x0"], cfg["y0"], z, dx, N, rows=(0, rows),
                          nthreads=threads)
    t1 = time.perf_counter() - t0
    rows2 = int(min(N, max(rows, rows * target_s / max(t1, 1e-3))))
    rows2 = max(threads, (rows2 // threads) * threads)
    t0 = time.perf_counter()
    ol.cpu_eval_plane_f32(ol.AXIS_XY, W32, begin, end, zl, cfg["x0"], cfg["y0"], z, dx, N, rows=(0, rows2),
                          nthreads=threads)
    t2 = time.perf_counter() - t0
    units = rows2 * N * int(counts[iz])
    return units / t2, threads, f"{rows2} rows x {N} points of the xy plane at z={z:.3f} ({counts[iz]} waves/point)"


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    cfg = CFG1
    fs, (Pi, zs, Pr, Pt), d = build_workload(cfg)
    W, begin, end, zl = unpack_arrays(Pi, zs, Pr, Pt)
    W32 = W.astype(np.complex64)
    rates = []
    sample = ""
    threads = None
    for i in range(args.warmup + args.steps):
        r, threads, sample = cpu_reference_rate(W32, begin, end, zl, cfg, d, target_s=args.ref_seconds)
        if i >= args.warmup:
            rates.append(r)
    v = float(np.mean(rates))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic", "impl": "reference",
            "config": {"workload": cfg["name"], "form": "reference FP32 CPU evaluator (cpu_cw_evaluate_xy)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from scwatter_gb300 import evaluator as ev
    from scwatter_gb300.cw import CoupledWaveStructure, HomogeneousLayer

    cfg = dict(CFG1)
    fs, (Pi, zs, Pr, Pt), d = build_workload(cfg)
    dx, dy, dz = d
    if args.nz:     # small profiling case: the central nz z-planes of the grid
        k0 = (cfg["Nz"] - args.nz) // 2
        cfg["z0"] = float(grid_axis(cfg["z0"], dz, cfg["Nz"])[k0])
        cfg["Nz"] = args.nz
        cfg["name"] += f" (central {args.nz} z-planes)"
    S = CoupledWaveStructure()
    S.Pi = Pi
    S.Layers = [HomogeneousLayer(z=zs[l], Pr=Pr[l], Pt=Pt[l]) for l in range(len(zs))]
    # a dedicated (non-default) stream: the context launches on it and the CUDA events
    # below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = ev.Context(local, stream=stream.cuda_stream)
    wset = ev.WaveSet.from_cw(ctx, S)
    W, begin, end, zl = unpack_arrays(Pi, zs, Pr, Pt)
    zgrid = grid_axis(cfg["z0"], dz, cfg["Nz"])
    counts = region_counts(begin, end, zl, 0, zgrid)
    units_per_step = int(counts.sum()) * cfg["Nx"] * cfg["Ny"]
    Nx, Ny, Nz = cfg["Nx"], cfg["Ny"], cfg["Nz"]
    out = torch.empty((Nz, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        wset.eval_volume_device(cfg["x0"], cfg["y0"], cfg["z0"], dx, dy, dz, Nx, Ny, Nz, out.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = ctx.launches
    times = []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.fill_(1.0)        # L2 flush between timed steps (outside the event pair)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    launches = ctx.launches - launches0
    clocks = sampler.stop()
    t_step = float(np.mean(times))
    if ws > 1:
        tt = torch.tensor([t_step], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_step = float(tt.item())
    value = units_per_step * ws / t_step

    # e2e: public host-buffer API: upload the float wave table from pinned host memory,
    # evaluate the volume, read the volume back.
    W32 = np.ascontiguousarray(W.astype(np.complex64))
    host_out = torch.empty((Nz, Ny, Nx, 3), dtype=torch.complex64, pin_memory=True)
    W_pinned = torch.from_numpy(W32.view(np.float32)).pin_memory()
    e2e_times = []
    for i in range(max(1, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w2 = ev.WaveSet.from_unpacked(ctx, len(zl), zl.astype(np.float32), begin, end,
                                      W_pinned.numpy().view(np.complex64))
        w2.eval_volume_device(cfg["x0"], cfg["y0"], cfg["z0"], dx, dy, dz, Nx, Ny, Nz, out.data_ptr())
        host_out.copy_(out, non_blocking=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        w2.close()
        if i > 0:
            e2e_times.append(dt)
    e2e_v = units_per_step / float(np.mean(e2e_times))

    # roofline: plain form is bound by the MUFU (SFU) pipe: 3 MUFU ops (ex2, sin, cos) per point*mode
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    peak_mufu = 16 * sm_count * sm_mhz * 1e6
    achieved_mufu = 3.0 * units_per_step / t_step
    line = None
    if rank == 0:
        cpu_v, cores, sample = cpu_reference_rate(W32, begin, end, zl, cfg, d, target_s=args.ref_seconds)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "c64", "data": "synthetic",
                "config": {"workload": cfg["name"], "form": "plain summation (FP64 tile re-base, FP32 MUFU)",
                           "points_modes_per_step": units_per_step, "l2": "flushed between timed steps"},
                "roofline": {"bound": "sfu", "achieved": achieved_mufu / 1e9, "peak": peak_mufu / 1e9,
                             "unit": "GMUFU/s", "frac": achieved_mufu / peak_mufu, "traffic": None,
                             "peak_source": f"16 MUFU/clk/SM x {sm_count} SMs x {sm_mhz:.0f} MHz (median under load)"},
                "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
                "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": int(W32.nbytes),
                        "d2h_bytes_per_step": int(Nx * Ny * Nz * 24)},
                "gpu_launches": int(launches), "clocks": clocks}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--nz", type=int, default=0, help="evaluate only this many z-planes (small profiling case)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
