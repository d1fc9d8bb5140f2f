#!/usr/bin/env python3
"""Throughput of the fused thin-film LBM step on GB300, as one JSON line.

Workload (Rayleigh-Taylor film, 512x512): g = -0.001, γ = 0.0005, θ = 1/9,
h0 = 1 + U[-0.01, 0.01] (seed 2), the Δh and mass series recorded every
time step (time_loop(sys, state, Δh), src/simulate.jl:47-67).  The hanging
film is linearly unstable: from this input the Float64 reference algorithm
diverges near t = 2300, so one benchmark step is a fresh simulation of 2000
time steps from h0 (state reset on the device), and the default 25 steps
add up to the configuration's 50,000 time steps.

  value      device time (CUDA events on the launching stream), inputs
             resident in HBM, L2 flushed (256 MiB write) between steps
  e2e        the same work through the reference-facing API with host
             buffers: state.height = h0 (host), time_loop, height back
  roofline   the fused step kernel: algorithmic bytes per launch (72 B per
             lattice update in FP32: 9 reads + 9 writes) over its average
             launch time, against the measured HBM copy bandwidth
  cpu_baseline  the oracle (Float64, fused, OpenMP on all host cores) on a
             bounded sample of the same workload

`--impl reference` times the CPU restatement of the reference algorithm
(Float64, all host threads) on the same configuration instead.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "swalbe.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

CHUNK = 2000  # time steps per benchmark step
B_ALG = {"f64": 144, "f32": 72, "f16": 40}  # bytes per lattice update: 9 reads + 9 writes


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=25)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="f32", choices=["f32", "f16", "f64"])
    ap.add_argument("--chunk", type=int, default=CHUNK)
    ap.add_argument("--no-extras", action="store_true", help="skip the 2048² and FP64 side runs")
    ap.add_argument("--profile-case", choices=["rt512", "film2048", "ensemble64"],
                    help="run a few steps of one case, untimed (for ncu captures)")
    ap.add_argument("--geometry", default="",
                    help="strip geometry NT,H (default: the autotuner's choice)")
    ap.add_argument("--step-mode", default="per_iteration", choices=["per_iteration", "multi"],
                    help="launch form for --profile-case")
    ap.add_argument("--case-steps", type=int, default=12)
    ap.add_argument("--mass-correction", default="default", choices=["default", "on", "off"],
                    help="mass controller of --profile-case (default: on for FP16 only)")
    ap.add_argument("--size", type=int, default=0, help="lattice side of --workload dewetting")
    ap.add_argument("--dry-run", action="store_true",
                    help="rank set-up and ensemble sharding only, no GPU work")
    ap.add_argument("--workload", choices=["ensemble", "serving", "spinodal", "lattice2048",
                                           "dewetting"],
                    help="print the ensemble, serving, spinodal-comparison or 2048² FP32/FP16 "
                         "line only")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def kernel_name(prec, geo, form):
    """The dominant kernel of a run with this geometry and launch form."""
    store = {"f32": "StoreF32", "f16": "StoreF16", "f64": "StoreF64"}[prec]
    if geo[0] == 33:
        return (f"resident_run_kernel<{store}> (tiles of 64x{geo[1]} in shared memory, up to "
                "1024 iterations per cooperative launch; figures per iteration)")
    if geo[0] < 0:
        return f"pair_step_kernel<{store}, {-geo[0]}> (pair strips of {-2 * geo[0] - 4}x{geo[1]})"
    if form == "multi":
        return f"fused_run_kernel<{store}, {256 if geo[0] == 32 else geo[0]}, {geo[0] == 32}>"
    if geo[0] == 32:
        return f"fused_tile_kernel<{store}> (2D tiles 32x16)"
    return f"fused_step_kernel<{store}, {geo[0]}> (strips of {geo[0] - 4}x{geo[1]})"


def load_traffic(kernel_key: str):
    """Per-launch DRAM bytes of the kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return d.get(kernel_key)
    except Exception:
        return None


def cpu_baseline(h0, sysc, chunk_steps=1000, chunks=4):
    """The oracle (Float64, fused, OpenMP) on a bounded sample of the workload."""
    import oracle
    oracle.build()
    p = sysc.param
    P = oracle.params(sysc.Lx, sysc.Ly, Tmax=chunk_steps, tdump=chunk_steps, tau=p.tau,
                      gamma=p.gamma, theta=p.theta, g=p.g, delta=p.delta, n=p.n, m=p.m,
                      hmin=p.hmin, hcrit=p.hcrit)
    threads = oracle.max_threads()
    t0 = time.perf_counter()
    for _ in range(chunks):
        oracle.FusedState(P, h0).run(chunk_steps, record_dh=True, nthreads=threads)
    dt = time.perf_counter() - t0
    lu = sysc.Lx * sysc.Ly * chunk_steps * chunks
    # the reference's own op sequence (one pass per op, one core): the closest
    # stand-in for its single-threaded Julia broadcasts
    lit_steps = 20
    t1 = time.perf_counter()
    oracle.time_loop_literal(P, h0, lit_steps, record_dh=True)
    dt1 = time.perf_counter() - t1
    return {"value": lu / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{chunks} x {chunk_steps} time steps of the {sysc.Lx}x{sysc.Ly} workload "
                      f"from h0, Float64, {dt:.1f} s",
            "literal_single_thread": {
                "value": sysc.Lx * sysc.Ly * lit_steps / dt1 / 1e6, "unit": "MLUPS", "cores": 1,
                "sample": f"{lit_steps} time steps, the literal per-op oracle, {dt1:.2f} s"}}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle
    from swalbe_gb300 import configs
    oracle.build()
    sysc, h0, _ = configs.rayleigh_taylor_512()
    p = sysc.param
    sample_steps = 100
    P = oracle.params(sysc.Lx, sysc.Ly, Tmax=sample_steps, tdump=sample_steps, tau=p.tau,
                      gamma=p.gamma, theta=p.theta, g=p.g)
    threads = oracle.max_threads()
    for _ in range(args.warmup):
        oracle.FusedState(P, h0).run(sample_steps, record_dh=True, nthreads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.FusedState(P, h0).run(sample_steps, record_dh=True, nthreads=threads)
        times.append(time.perf_counter() - t0)
    lu = sysc.Lx * sysc.Ly * sample_steps
    value = lu * len(times) / sum(times) / 1e6
    line = {
        "impl": "reference", "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "rayleigh_taylor_512: 512x512, g=-0.001, gamma=0.0005, theta=1/9, "
                               "h0=1+U[-0.01,0.01] seed 2",
                   "sample": f"{sample_steps} time steps from h0 per step"},
        "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": f"{sample_steps} time steps of 512x512 per step, Float64, "
                                   "oracle restatement of the Julia reference (Julia is absent)"},
        "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def timed_chunks(st, sw, torch, stream, d_h0, d_zero, flush, K, chunk, N):
    """K benchmark steps; returns (per-step ms list, per-launch kernel ms list)."""
    step_ms, launch_ms = [], []
    for _ in range(K):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        k0 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st.set_device("height", d_h0.data_ptr())
        st.set_device("velx", d_zero.data_ptr())
        st.set_device("vely", d_zero.data_ptr())
        k0.record(stream)
        st.step(chunk)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        launch_ms.append(k0.elapsed_time(e1) / chunk)
        st.measures()  # drain the Δh/mass records (outside the events)
    return step_ms, launch_ms


def run_ours(args):
    import numpy as np
    import torch

    import swalbe_gb300 as sw
    from swalbe_gb300 import _lib as L
    from swalbe_gb300 import configs

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        if rank == 0:
            print(f"ranks: {dist.get_world_size()} (nccl)", file=sys.stderr, flush=True)
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    sw.build()
    T = {"f32": np.float32, "f16": np.float16, "f64": np.float64}[args.precision]
    sysc, h0, total = configs.rayleigh_taylor_512()
    N = sysc.Lx * sysc.Ly
    chunk = args.chunk
    stream = torch.cuda.Stream()
    st = sw.Sys(sysc, "GB300", T=T)
    st.set_stream(stream.cuda_stream)
    st.set_theta(sysc.param.theta)
    st.set_measures(L.MEAS_MASS | L.MEAS_MAXMIN)
    if args.geometry:  # a fixed geometry instead of the autotuner (e.g. for ncu captures)
        st.set_geometry(*(int(v) for v in args.geometry.split(",")))
    d_h0 = torch.from_numpy(np.ascontiguousarray(h0.ravel(order="F"))).to(f"cuda:{dev}")
    d_zero = torch.zeros(N, dtype=torch.float64, device=f"cuda:{dev}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    torch.cuda.synchronize()

    # warm-up (graph capture, clocks)
    timed_chunks(st, sw, torch, stream, d_h0, d_zero, flush, args.warmup, chunk, N)

    clocks = ClockSampler(dev)
    clocks.start()
    n0 = sw.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    torch.cuda.nvtx.range_push("timed")  # the launch-list capture filters on this range
    step_ms, launch_ms = timed_chunks(st, sw, torch, stream, d_h0, d_zero, flush, args.steps,
                                      chunk, N)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    if world > 1:
        torch.distributed.barrier()
    launches = sw.launch_count() - n0
    clk = clocks.stop()
    geo, form = st.geometry(), st.step_mode()

    dev_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([dev_s], device=f"cuda:{dev}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_s = float(t.item())
    lu_rank = N * chunk * args.steps
    value = world * lu_rank / dev_s / 1e6

    # result check: the first chunk against the GPU Float64 path
    st.set_device("height", d_h0.data_ptr())
    st.set_device("velx", d_zero.data_ptr())
    st.set_device("vely", d_zero.data_ptr())
    st.step(chunk)
    h_ours = st.height
    st.measures()
    ref64 = sw.Sys(sysc, "GB300", T=np.float64)
    ref64.height = h0
    ref64.step(chunk)
    h_ref = ref64.height
    rel = float(np.linalg.norm(h_ours - h_ref) / np.linalg.norm(h_ref))
    rel_dev = float(np.linalg.norm(h_ours - h_ref) / np.linalg.norm(h_ref - 1.0))
    del ref64

    # e2e: reference-facing API with host buffers
    st.set_stream(None)
    e2e_sys = sw.SysConst(sysc.Lx, sysc.Ly, sysc.param.replace(Tmax=chunk, tdump=chunk))

    def pinned():  # a column-major Lx x Ly Float64 array in pinned host memory
        return torch.empty((sysc.Ly, sysc.Lx), dtype=torch.float64, pin_memory=True).numpy().T

    h_in, zeros, h_out = pinned(), pinned(), pinned()
    h_in[...] = h0
    zeros[...] = 0.0
    e2e_times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st.height = h_in
        st.velx = zeros
        st.vely = zeros
        diff = []
        sw.time_loop(e2e_sys, st, diff)
        st.get("height", out=h_out)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            e2e_times.append(dt)
    e2e_value = world * N * chunk * len(e2e_times) / sum(e2e_times) / 1e6

    hbm, peak_kind = peaks()
    t_launch = statistics.median(launch_ms) / 1e3
    alg_bytes = B_ALG[args.precision] * N
    achieved = alg_bytes / t_launch / 1e9
    key = (f"resident_{args.precision}_512" if geo[0] == 33 else
           f"pair_{args.precision}_512" if geo[0] < 0 else f"fused_step_{args.precision}_512")
    traffic = load_traffic(key)

    extras = {}
    if not args.no_extras and world > 1:
        extras["ensemble"] = ensemble_run(sw, np, rank=rank, world=world, torch=torch)
    if not args.no_extras and world == 1:
        extras = side_runs(sw, L, np, torch, hbm)
        extras["ensemble"] = ensemble_run(sw, np)
        extras["serving"] = serving_run(sw, np)
        # spinodal dewetting, bounded: 2048², 10,000 steps in each precision
        extras["dewetting_2048"] = dewetting_run(sw, np, L, n=2048, steps=10000)

    line = {
        "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(step_ms) / len(step_ms),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": args.precision, "data": "synthetic",
        "config": {
            "workload": "rayleigh_taylor_512: 512x512 thin film, g=-0.001, gamma=0.0005, "
                        "theta=1/9, tau=1, h0=1+U[-0.01,0.01] seed 2; Δh and mass every time step",
            "time_steps_per_step": chunk, "total_time_steps": chunk * args.steps,
            "precision": {"f32": "FP32 arithmetic, FP32 populations",
                          "f16": "FP32 arithmetic, FP32 f0 + FP16 f1..f8",
                          "f64": "Float64 arithmetic (reference operation order)"}[args.precision],
            "l2": "flushed between timed steps (256 MiB write); the 512x512 state (19 MB) is "
                  "L2-resident within a step",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "geometry": {"nt": geo[0], "rows": geo[1], "form": form,
                         "chosen_by": "--geometry" if args.geometry else
                                       "autotuner (timed on the first 2000-step chunk)"},
        },
        "e2e": {"value": e2e_value, "unit": "MLUPS",
                # the reference-facing API takes and returns Float64 host
                # arrays (converted on the device); records are 56 bytes
                "h2d_bytes_per_step": 3 * N * 8,
                "d2h_bytes_per_step": N * 8 + chunk * 56,
                "host_buffers": "pinned"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "kernel": f"{kernel_name(args.precision, geo, form)}, 512x512, "
                               f"{B_ALG[args.precision]} B/LU algorithmic",
                     "launch_us": t_launch * 1e6, "peak_kind": f"{peak_kind} (hbm_gbs burst)"},
        "clocks": clk,
        "wall_s": wall,
        "check": {"vs": "GPU Float64 path (bit-identical to the oracle)", "after_time_steps": chunk,
                  "rel_l2_h": rel, "rel_l2_h_minus_1": rel_dev},
    }
    line.update(extras)
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline(h0, sysc)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def lattice_2048_run(sw, np, torch, hbm, precs=("f32", "f16", "f64"), geometry=""):
    """HBM-bound 2048² runs (the state is larger than L2), event-timed on the
    state's stream; `geometry` "NT,H" overrides the size rule's strips.
    FP32 also end to end (time_loop with pinned Float64 host buffers: h, ux,
    uy up and h down every call) and against Float64 after the same
    iterations (relative L2 of h)."""
    out = {}
    rng = np.random.default_rng(3)
    n = 2048
    h0 = np.asfortranarray(1.0 + rng.uniform(-0.1, 0.1, (n, n)))
    s2 = sw.SysConst(n, n, sw.Taumucs())
    h_f32 = None
    total_f32 = 0
    # f16_no_controller: FP16 storage with its mass controller off (on by
    # default: FP16 cannot hold the rounding residue, and the controller's
    # exact per-step mass sum costs ~7 % of the step)
    for prec, T, steps in (("f32", np.float32, 300), ("f16", np.float16, 300),
                           ("f16_no_controller", np.float16, 300), ("f64", np.float64, 30)):
        if prec.split("_")[0] not in precs:
            continue
        st = sw.Sys(s2, "GB300", T=T)
        if prec == "f16_no_controller":
            st.set_mass_correction(False)
        if geometry:
            st.set_geometry(*(int(v) for v in geometry.split(",")))
        stream = torch.cuda.Stream()
        st.set_stream(stream.cuda_stream)
        st.height = h0
        st.step(64)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st.step(steps)
        e1.record(stream)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / steps
        ach = B_ALG[prec.split("_")[0]] * n * n / t / 1e9
        line = {"MLUPS": n * n / t / 1e6, "launch_us": t * 1e6, "achieved_GBs": ach,
                "frac": ach / hbm, "geometry": list(st.geometry())}
        if prec == "f32":
            h_f32, total_f32 = st.height, 64 + steps
            line["e2e"] = lattice_2048_e2e(sw, np, torch, st, s2, h0)
        if prec == "f64" and h_f32 is not None:
            st.step(total_f32 - 64 - steps)
            h64 = st.height
            line_f32 = out["lattice_2048"]["f32"]
            line_f32["check"] = {
                "vs": "GPU Float64 path (bit-identical to the oracle)",
                "after_time_steps": total_f32,
                "rel_l2_h": float(np.linalg.norm(h_f32 - h64) / np.linalg.norm(h64)),
                "rel_l2_h_minus_1": float(np.linalg.norm(h_f32 - h64) / np.linalg.norm(h64 - 1.0))}
        out.setdefault("lattice_2048", {})[prec] = line
        del st
    return out


def lattice_2048_e2e(sw, np, torch, st, sysc, h0, calls=5, tmax=300):
    """MLUPS through time_loop with pinned Float64 host buffers (h, ux, uy
    uploaded and h downloaded every call, inside the timed region)."""
    def pinned():
        return torch.empty((sysc.Ly, sysc.Lx), dtype=torch.float64, pin_memory=True).numpy().T

    h_in, zeros, h_out = pinned(), pinned(), pinned()
    h_in[...] = h0
    zeros[...] = 0.0
    e2e_sys = sw.SysConst(sysc.Lx, sysc.Ly, sysc.param.replace(Tmax=tmax, tdump=tmax))
    st.set_stream(None)
    times = []
    for k in range(calls + 1):
        t0 = time.perf_counter()
        st.height = h_in
        st.velx = zeros
        st.vely = zeros
        sw.time_loop(e2e_sys, st)
        st.get("height", out=h_out)
        if k > 0:  # the first call warms up
            times.append(time.perf_counter() - t0)
    nb = sysc.Lx * sysc.Ly * 8
    return {"MLUPS": sysc.Lx * sysc.Ly * tmax * len(times) / sum(times) / 1e6,
            "time_steps_per_call": tmax, "h2d_bytes_per_call": 3 * nb, "d2h_bytes_per_call": nb,
            "host_buffers": "pinned"}


def side_runs(sw, L, np, torch, hbm):
    """HBM-bound 2048² runs and the Float64 paths."""
    out = lattice_2048_run(sw, np, torch, hbm)
    s5 = sw.SysConst(512, 512, sw.Taumucs(g=-0.001, gamma=0.0005))
    h5 = np.asfortranarray(1.0 + np.random.default_rng(2).uniform(-0.01, 0.01, (512, 512)))
    for dev_name, steps in (("GB300", 200), ("GB300-plain", 50)):
        st = sw.Sys(s5, dev_name, T=np.float64)
        st.height = h5
        st.step(10)
        st.sync()
        t0 = time.perf_counter()
        st.step(steps)
        st.sync()
        dt = time.perf_counter() - t0
        out.setdefault("fp64_512", {})["fused" if dev_name == "GB300" else "plain"] = {
            "MLUPS": 512 * 512 * steps / dt / 1e6}
        del st
    return out


def ensemble_run(sw, np, count=512, steps=200, plain_sample=8, geometry="", rank=0, world=1,
                 torch=None):
    """Coalescence ensemble: `count` two-cap lattices (128², 256², 512²,
    1024x256) advanced together in FP32 by the batch kernel, against the
    plain one-at-a-time paths on a sample of the same instances.  With
    `world` ranks each rank advances its round-robin share of the members
    (configs.shard; no data moves between ranks) and the line reports all
    members' lattice updates over the slowest rank's time."""
    from swalbe_gb300 import configs
    members, full_steps = configs.ensemble(count)
    if world > 1:
        members = configs.shard(members, rank, world)
    systems = [m.sysc for m in members]
    cells = sum(s.Lx * s.Ly for s in systems)
    b = sw.Batch(systems, T=np.float32)
    if geometry:  # a fixed strip geometry (the tuner then picks only the CTA count)
        b.set_geometry(*(int(v) for v in geometry.split(",")))
    for i, m in enumerate(members):
        b.set_height(i, m.h0)
    b.step(40)  # includes the autotuning probes
    b.sync()
    t0 = time.perf_counter()
    b.step(steps)
    b.sync()  # raises if any lattice went non-finite
    dt = time.perf_counter() - t0
    local_cells = cells
    if world > 1:  # every rank's cells over the slowest rank's time
        dev = torch.cuda.current_device()
        t = torch.tensor([dt], device=f"cuda:{dev}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        c = torch.tensor([float(cells)], device=f"cuda:{dev}", dtype=torch.float64)
        torch.distributed.all_reduce(c)
        dt, cells = float(t.item()), int(c.item())
    batch_mlups = cells * steps / dt / 1e6
    tile = b.tile()
    bgeo = b.geometry()
    b.close()
    del b
    if world > 1:
        return {"instances": count, "cells": cells, "time_steps_per_sim": full_steps,
                "batch_f32": {"MLUPS": batch_mlups, "sims_per_s": count * steps / (dt * full_steps),
                              "timed_steps": steps},
                "shard": {"ranks": world, "members_on_rank0": len(members),
                          "cells_on_rank0": local_cells, "split": "round robin (configs.shard)"}}
    # one at a time: the plain Float64 per-op path and the fused FP32 step
    rng = np.random.default_rng(0)
    sample = [members[i] for i in rng.choice(len(members), plain_sample, replace=False)]
    out = {}
    for label, dev, T, nst in (("plain_f64_one_at_a_time", "GB300-plain", np.float64, 30),
                               ("fused_f32_one_at_a_time", "GB300", np.float32, 200)):
        lu, tt = 0.0, 0.0
        for m in sample:
            st = sw.Sys(m.sysc, dev, T=T)
            st.height = m.h0
            st.step(5)
            st.sync()
            t1 = time.perf_counter()
            st.step(nst)
            st.sync()
            tt += time.perf_counter() - t1
            lu += m.sysc.Lx * m.sysc.Ly * nst
            del st
        out[label] = {"MLUPS": lu / tt / 1e6, "sample": f"{plain_sample} instances x {nst} steps"}
    return {
        "instances": count, "cells": cells, "time_steps_per_sim": full_steps,
        "batch_f32": {"MLUPS": batch_mlups, "sims_per_s": count * steps / (dt * full_steps),
                      "timed_steps": steps, "strip": {"width": tile[0], "rows": tile[1],
                                "threads": abs(bgeo[0]), "columns_per_thread": 2 if bgeo[0] < 0 else 1,
                                "ctas": bgeo[2], "chosen_by": "batch autotuner (strip shapes x CTA counts)"}},
        **out,
        "speedup_vs_plain": batch_mlups / out["plain_f64_one_at_a_time"]["MLUPS"],
        "speedup_vs_fused_one_at_a_time": batch_mlups / out["fused_f32_one_at_a_time"]["MLUPS"],
    }


def serving_run(sw, np, duration=12.0, rate=200.0, budget=24 << 30, steps_per_tick=100,
                queue_limit=256, policy="sjf", max_cells=16 << 20, geometry=None):
    """Poisson arrivals (200/s) of thin-film solves (sides 64..2048, 1k-100k
    steps, moving wettability, g in [-1e-3, 0]) into the server for
    `duration` seconds.  The offered load is ~300x what one GPU serves, so
    the queue is bounded; shortest-job-first admission with a bound on the
    resident cells keeps lock-step ticks short (~60 ms), and a full queue
    sheds its largest job."""
    from swalbe_gb300 import configs
    reqs = configs.serving_stream(rate=rate, duration=duration, seed=5)
    sv = sw.Server(budget, T=np.float32, steps_per_tick=steps_per_tick)
    sv.set_queue_limit(queue_limit)
    sv.set_policy(policy, max_cells)
    if geometry:  # (nt, rows): fixed strips instead of the server's choice
        sv.set_geometry(*geometry)
    t0 = time.perf_counter()
    pending, done, rejected, i = {}, [], 0, 0
    sizes, failed = [], {}
    offered_lu = 0.0
    while True:
        now = time.perf_counter() - t0
        while i < len(reqs) and reqs[i].t_arrival <= now:
            r = reqs[i]
            i += 1
            offered_lu += r.sysc.Lx * r.sysc.Ly * r.nsteps
            rid = sv.submit(r.sysc, r.height(), r.nsteps, theta0=r.theta0, dtheta=r.dtheta, v=r.v)
            if rid is None:
                rejected += 1
            else:
                pending[rid] = r
        for rid in list(pending):
            ok, _, info = sv.poll(rid)
            if ok:
                done.append(info.t_done - info.t_submit)
                sizes.append(pending[rid].sysc.Lx * pending[rid].sysc.Ly * pending[rid].nsteps)
                del pending[rid]
            elif info.status < 0:  # shed from a full queue, or failed
                failed[info.status] = failed.get(info.status, 0) + 1
                del pending[rid]
        if now > duration:
            break
        time.sleep(0.002)
    st = sv.stats()
    wall = time.perf_counter() - t0
    # requests still queued or resident when the window closes: their
    # latency is at least the time they have waited so far (censored)
    t_end = sv.clock()
    censored = []
    for rid in pending:
        _, _, info = sv.poll(rid)
        if info.status >= 0:
            censored.append(t_end - info.t_submit)
    lat = sorted(done)
    pct = (lambda q: lat[min(len(lat) - 1, int(q * len(lat)))] if lat else None)
    every = sorted(done + censored)
    pct_all = (lambda q: every[min(len(every) - 1, int(q * len(every)))] if every else None)
    res = {
        "duration_s": wall, "offered_req_per_s": rate, "arrivals": i,
        "offered_MLUPS": offered_lu / duration / 1e6,
        "served_MLUPS": st.lattice_updates / wall / 1e6,
        "ticks": int(st.ticks), "tick_busy_s": st.busy_seconds, "device_s": st.device_seconds,
        "device_MLUPS": st.lattice_updates / st.device_seconds / 1e6 if st.device_seconds else None,
        "completed": len(done), "admitted": int(st.admitted), "rejected_queue_full": rejected,
        "resident_at_end": int(st.running), "queued_at_end": int(st.queued),
        "latency_s": {"p50": pct(0.50), "p99": pct(0.99), "max": lat[-1] if lat else None,
                      "over": "completed requests"},
        "latency_all_arrivals_s": {
            "p50": pct_all(0.50), "p99": pct_all(0.99), "completed": len(done),
            "censored": len(censored),
            "over": "every admitted or queued arrival; one unfinished at the window end counts "
                    "its wait so far (a lower bound)"},
        "hbm_budget_GB": budget / 1e9, "steps_per_tick": steps_per_tick,
        "policy": policy, "max_resident_cells": max_cells, "queue_limit": queue_limit,
        "shed_or_rejected_total": int(st.rejected),
        "ended_with_status": {str(k): v for k, v in failed.items()},
        "completed_work_LU": {"median": float(np.median(sizes)) if sizes else None,
                              "max": float(max(sizes)) if sizes else None},
    }
    sv.close()
    return res


def dewetting_run(sw, np, L_, n=2048, steps=10000):
    """The dewetting film (configs.dewetting_film: h0 = 0.2 (1 + U[-0.1,
    0.1]), θ = 1/9, n²): Float64, FP32 and FP16-storage runs after `steps`
    iterations: droplets (h > 0.055, periodic 8-connected), relative L2 of h
    against Float64, mass drift."""
    from swalbe_gb300 import configs
    sysc, h0, _ = configs.dewetting_film(n=n)
    out = {"steps": steps, "lattice": [n, n], "film": "h0 = 0.2 (1 + U[-0.1, 0.1]), seed 3, "
           "theta = 1/9, gamma = 0.01: ruptures into droplets"}
    res = {}
    for name, T in (("f64", np.float64), ("f32", np.float32), ("f16", np.float16)):
        st = sw.Sys(sysc, "GB300", T=T)
        st.set_measures(L_.MEAS_MASS)
        st.height = h0
        t0 = time.perf_counter()
        masses, done = [], 0
        while done < steps:
            k = min(L_.RECORD_CAPACITY, steps - done)
            st.step(k)
            masses += [r.mass for r in st.measures(cap=k)]
            done += k
        st.sync()
        dt = time.perf_counter() - t0
        h = st.height
        m = np.array(masses)
        res[name] = h
        out[name] = {"seconds": dt, "MLUPS": n * n * steps / dt / 1e6,
                     "droplets": sw.count_droplets(h), "hmax": float(h.max()),
                     "mass_drift_max": float(np.abs(m - m[0]).max() / m[0])}
        del st
    ref = res["f64"]
    for name in ("f32", "f16"):
        out[name]["rel_l2_h_vs_f64"] = float(np.linalg.norm(res[name] - ref) / np.linalg.norm(ref))
        out[name]["droplets_vs_f64"] = out[name]["droplets"] - out["f64"]["droplets"]
    return out


def spinodal_run(sw, np, L_, steps=100000):
    """The spinodal-comparison film, 2048² (h = 1 + U[-0.1, 0.1], seed 3,
    γ = 0.01, θ = 1/9): FP32 and FP16-storage runs against the Float64 run
    of the same film, after `steps` iterations: relative L2 of h, mass drift
    (FP64 sums of the per-iteration mass), droplets (h > 0.055, periodic
    8-connected)."""
    from swalbe_gb300 import configs
    sysc, h0, _ = configs.spinodal_2048()
    out = {"steps": steps, "lattice": [sysc.Lx, sysc.Ly]}
    res = {}
    for name, T in (("f64", np.float64), ("f32", np.float32), ("f16", np.float16)):
        st = sw.Sys(sysc, "GB300", T=T)
        st.set_measures(L_.MEAS_MASS)
        st.height = h0
        t0 = time.perf_counter()
        done, masses = 0, []
        while done < steps:
            n = min(20000, steps - done)
            st.step(n)
            masses += [r.mass for r in st.measures()]
            done += n
        st.sync()
        dt = time.perf_counter() - t0
        h = st.height
        m = np.array(masses)
        res[name] = h
        out[name] = {"seconds": dt, "MLUPS": sysc.Lx * sysc.Ly * steps / dt / 1e6,
                     "mass_drift_max": float(np.abs(m - m[0]).max() / m[0]),
                     "droplets": sw.count_droplets(h), "hmax": float(h.max()),
                     "hmin": float(h.min())}
        del st
    ref = res["f64"]
    for name in ("f32", "f16"):
        out[name]["rel_l2_h_vs_f64"] = float(np.linalg.norm(res[name] - ref) / np.linalg.norm(ref))
    return out


def run_workload(args):
    import numpy as np

    import swalbe_gb300 as sw
    from swalbe_gb300 import _lib as L_
    sw.build()
    if args.workload == "spinodal":
        r = spinodal_run(sw, np, L_, steps=args.case_steps if args.case_steps != 12 else 100000)
        print(json.dumps({"workload": "spinodal_2048", **r}), flush=True)
        return
    if args.workload == "dewetting":
        n = args.size or 2048
        r = dewetting_run(sw, np, L_, n=n, steps=args.case_steps if args.case_steps != 12 else 10000)
        print(json.dumps({"workload": "dewetting", **r}), flush=True)
        return
    if args.workload == "lattice2048":
        import torch
        r = lattice_2048_run(sw, np, torch, peaks()[0], precs=("f32", "f16"),
                             geometry=args.geometry)
        print(json.dumps({"workload": "lattice_2048", **r}), flush=True)
        return
    if args.workload == "ensemble":
        r = ensemble_run(sw, np, geometry=args.geometry)
        line = {"metric": "MLUPS", "value": r["batch_f32"]["MLUPS"], "unit": "MLUPS",
                "workload": "ensemble", **r}
    else:
        r = serving_run(sw, np)
        line = {"metric": "MLUPS", "value": r["served_MLUPS"], "unit": "MLUPS",
                "workload": "serving", **r}
    print(json.dumps(line), flush=True)


def profile_case(args):
    """A few launches of one workload, untimed: the committed command that the
    ncu summaries under profiles/ were captured from."""
    import numpy as np

    import swalbe_gb300 as sw
    from swalbe_gb300 import _lib as L
    from swalbe_gb300 import configs
    sw.build()
    T = {"f32": np.float32, "f16": np.float16, "f64": np.float64}[args.precision]
    if args.profile_case == "ensemble64":
        # the first 64 members of the coalescence ensemble, batched (~0.7 GB)
        members, _ = configs.ensemble(64)
        b = sw.Batch([m.sysc for m in members], T=T)
        if args.geometry:  # e.g. -64,32: the pair strips the autotuner picks for the ensemble
            nt, hh = (int(v) for v in args.geometry.split(","))
            b.set_geometry(nt, hh)
        for i, m in enumerate(members):
            b.set_height(i, m.h0)
        b.step(args.case_steps)
        b.sync()
        tx, ty, spg = b.tile()
        print(json.dumps({"case": args.profile_case, "precision": args.precision,
                          "lattices": len(members), "cells": sum(m.sysc.Lx * m.sysc.Ly for m in members),
                          "strip": [tx, ty], "geometry": list(b.geometry()), "steps": args.case_steps}))
        b.close()
        return
    if args.profile_case == "rt512":
        sysc, h0, _ = configs.rayleigh_taylor_512()
        meas = L.MEAS_MASS | L.MEAS_MAXMIN
    else:
        n = 2048
        sysc = sw.SysConst(n, n, sw.Taumucs())
        h0 = np.asfortranarray(1.0 + np.random.default_rng(3).uniform(-0.1, 0.1, (n, n)))
        meas = 0
    st = sw.Sys(sysc, "GB300", T=T)
    if meas:
        st.set_measures(meas)
    if args.geometry:
        nt, hh = (int(v) for v in args.geometry.split(","))
        st.set_geometry(nt, hh)
    else:
        st.set_geometry(0, 0)
    st.set_step_mode(args.step_mode)
    if args.mass_correction != "default":
        st.set_mass_correction(args.mass_correction == "on")
    st.height = h0
    st.step(args.case_steps)
    st.sync()
    print(json.dumps({"case": args.profile_case, "precision": args.precision,
                      "geometry": st.geometry(), "form": st.step_mode(),
                      "mass_correction": args.mass_correction, "steps": args.case_steps}))


def launch_ranks(args) -> int:
    """`--gpus N` outside a launcher: run this script as N local ranks
    (torch.distributed.run, one process per GPU, rendezvous on 127.0.0.1)."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={args.gpus}", "--master-addr=127.0.0.1", f"--master-port={port}",
           os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def dry_run(args):
    """The rank set-up and the ensemble sharding without GPU work (on CPU
    ranks the process group uses gloo): rank 0 prints the rank count, the
    backend and every rank's ensemble members."""
    import torch
    import torch.distributed as dist
    rank, world, _ = dist_env()
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if world > 1:
        dist.init_process_group(backend)
    from swalbe_gb300 import configs
    mine = configs.shard(list(range(512)), rank, world)
    shards = [mine]
    if world > 1:
        shards = [None] * world
        dist.all_gather_object(shards, mine)
    if rank == 0:
        print(json.dumps({"dry_run": True, "n_gpus": world, "backend": backend,
                          "ensemble_shards": shards}), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args))
    if args.dry_run:
        dry_run(args)
        return
    if args.profile_case:
        profile_case(args)
        return
    if args.workload:
        run_workload(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
