#!/usr/bin/env python3
"""Benchmark of the GB300 rough Bergomi RT pricer.

Default workload (the configuration the headline metric is quoted on):
mixed precision, H = 0.1, eta = 1.9, rho = -0.9, xi = 0.235^2, T = 1,
21 strikes on [0.6, 1.4], N = 512 steps, M = 2^22 paths, Philox seed 11.
One step = one full pricing call over all M paths.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints ONE JSON line.  `value` is path-steps/s (path x step x distinct H) of
the mixed form timed with CUDA events on the launching stream, L2 flushed
(256 MiB write) before every timed step.  `e2e` is the same metric through
the drop-in C-ABI call computeIVRT_tensor with host buffers.  The FP64 form
is timed on the same workload, and the mixed prices are compared with the
FP64 form on identical normals.  At one GPU the line also carries a
`serving` object: the 10,000-request Poisson stream (200 requests/s, mixed
parameters, N and M log-uniform) replayed through the serving loop, with
p50 / p99 / max latency, prices/s and path-steps/s delivered, the sampled
clocks of that window, and the plain FP64 form one request at a time on a
sample of the same stream (`--skip-serving` leaves it out).
`--impl reference` times the CPU oracle (the C restatement of the
reference's OpenMP path) on a bounded sample of the same workload on all
host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "mixed-n512-m4m-21k": dict(xi=0.235 ** 2, H=[0.1], eta=[1.9], rho=[-0.9], T=[1.0] * 21,
                               K=[round(float(k), 10) for k in np.linspace(0.6, 1.4, 21)], N=512, M=1 << 22,
                               seed=11),
    # long-horizon crossover sweep shape: three H, T = 2, 11 strikes on [0.5, 1.5], M = 2^20, seed 3
    "mixed-crossover-m1m-11k": dict(xi=0.04, H=[0.03, 0.1, 0.4], eta=[1.5] * 3, rho=[-0.7] * 3, T=[2.0] * 11,
                                    K=[round(float(k), 10) for k in np.linspace(0.5, 1.5, 11)], N=1024,
                                    M=1 << 20, seed=3),
    "fp64-n100-m64k-5k": dict(xi=0.235 ** 2, H=[0.07], eta=[1.9], rho=[-0.9], T=[1.0] * 5,
                              K=[0.8, 0.9, 1.0, 1.1, 1.2], N=100, M=1 << 16, seed=42),
}
DEFAULT = "mixed-n512-m4m-21k"
METRIC = "path-steps/s"


def path_steps(w) -> float:
    return float(w["M"]) * w["N"] * len(set(w["H"]))


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# --------------------------------------------------------------- CPU arm
def cpu_sample(w, paths: int, threads: int):
    """Times the oracle's C restatement of the reference RT path (OpenMP over
    paths, FP64, direct causal Volterra sum) on `paths` paths of workload w."""
    from oracle import oracle as O
    O.lib()
    t0 = time.perf_counter()
    O.price_rt_philox(w["xi"], w["H"], w["eta"], w["rho"], w["T"], w["K"], w["N"], paths, w["seed"], threads)
    dt = time.perf_counter() - t0
    return paths * w["N"] * len(set(w["H"])) / dt, dt


def run_reference(args, w):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.lib()
    threads = O.max_threads()
    paths = args.cpu_paths
    for _ in range(args.warmup):
        cpu_sample(w, paths, threads)
    vals = []
    t_all = 0.0
    for _ in range(args.steps):
        v, dt = cpu_sample(w, paths, threads)
        vals.append(v)
        t_all += dt
    value = args.steps * paths * w["N"] * len(set(w["H"])) / t_all
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "path-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_all / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "N": w["N"], "M_sample_per_step": paths, "strikes": len(w["K"]),
                   "note": "CPU oracle: C restatement of rBergLib's RT path (direct causal sum in place of FFTW)"},
        "cpu_baseline": {"value": value, "unit": "path-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{paths} paths x N={w['N']} per step"},
        "e2e": {"value": value, "unit": "path-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# --------------------------------------------------------------- GPU arm
class _Nvml:
    """Read-only NVML queries through ctypes (libnvidia-ml is installed with the GPU kernel driver):
    SM clock, its maximum, board power and the active clock-event reasons of one
    GPU, found by the PCI bus id CUDA reports for the device."""

    SM = 1  # NVML_CLOCK_SM
    # nvmlClocksEventReasons bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, cuda_index: int):
        import ctypes
        import torch
        self.c = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.lib = lib
        pr = torch.cuda.get_device_properties(cuda_index)
        bus = f"{pr.pci_domain_id:08X}:{pr.pci_bus_id:02X}:{pr.pci_device_id:02X}.0".encode()
        self.dev = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(self.dev)) != 0:
            lib.nvmlShutdown()
            raise OSError(f"no NVML device at {bus.decode()}")
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        u = ctypes.c_uint()
        self.max_mhz = float(u.value) if lib.nvmlDeviceGetMaxClockInfo(self.dev, self.SM, ctypes.byref(u)) == 0 \
            else None

    def sample(self):
        c, lib = self.c, self.lib
        mhz, mw, rs = c.c_uint(), c.c_uint(), c.c_ulonglong()
        if lib.nvmlDeviceGetClockInfo(self.dev, self.SM, c.byref(mhz)) != 0:
            return None
        watts = mw.value / 1e3 if lib.nvmlDeviceGetPowerUsage(self.dev, c.byref(mw)) == 0 else None
        bits = rs.value if self.reasons_fn(self.dev, c.byref(rs)) == 0 else 0
        return float(mhz.value), watts, [n for b, n in self.REASONS.items() if bits & b]

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """SM clock, power and throttle reasons sampled while the timed region runs:
    NVML every 10 ms on a thread, or `nvidia-smi -lms 200` where NVML cannot be
    loaded."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    SMI_REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.nvml = None
        self.rows = []  # (sm MHz, max MHz, watts or None, [active reasons])
        self.source = None

    def _poll(self):
        while not self.stop.wait(0.01):
            s = self.nvml.sample()
            if s:
                self.rows.append((s[0], self.nvml.max_mhz, s[1], s[2]))

    def __enter__(self):
        import threading
        try:
            self.nvml = _Nvml(self.index)
        except Exception:
            self.nvml = None
        if self.nvml is not None:
            self.source = "nvml 10 ms"
            s = self.nvml.sample()
            if s:
                self.rows.append((s[0], self.nvml.max_mhz, s[1], s[2]))
            self.stop = threading.Event()
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.source = "nvidia-smi 200 ms"
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml is not None:
            self.stop.set()
            self.thread.join()
            s = self.nvml.sample()
            if s:
                self.rows.append((s[0], self.nvml.max_mhz, s[1], s[2]))
            self.nvml.close()
            return
        out = ""
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
        for line in (out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                self.rows.append((float(parts[1]), float(parts[2]), float(parts[3]),
                                  [n for n, v in zip(self.SMI_REASONS, parts[4:8]) if v.lower() == "active"]))
            except ValueError:
                continue

    def summary(self):
        rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        active = sorted({n for r in rows for n in r[3]})
        loaded = [r for r in rows if r[2] is not None and r[2] > 200.0] or rows
        maxes = [r[1] for r in rows if r[1] is not None]
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": max(maxes) if maxes else None,
                "reasons": active, "samples": len(rows), "source": self.source}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, 6800.0, "fallback"


def kernel_figure(kernel: str, key: str):
    """A per-kernel figure from the committed ncu summaries (profiles/traffic.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)[kernel][key]
    except (OSError, KeyError, ValueError, TypeError):
        return None


def issue_roofline(kernel: str, path_steps_per_launch: float, kernel_ms: float, clocks: dict):
    """The binding resource of the mixed path kernels is instruction issue:
    ncu's thread-instructions per path-step (profiles/traffic.json) times the
    live kernel rate, in warp-instructions/s, against one issue per cycle per
    SM sub-partition (4 per SM) at the SM clock sampled during the run."""
    ips = kernel_figure(kernel, "inst_per_path_step")
    mhz = clocks.get("sm_mhz") if clocks else None
    if ips is None or not mhz:
        return None
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    achieved = path_steps_per_launch / (kernel_ms / 1e3) * ips / 32.0
    peak = 4.0 * sms * mhz * 1e6
    return {"unit": "warp-instr/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "inst_per_path_step": ips, "source": "ncu smsp__inst_executed (profiles), live kernel time, sampled clock"}


def traffic_per_launch(kernel: str, w):
    """DRAM bytes per launch from the committed ncu summary, scaled by paths."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)[kernel]
        return d["bytes"] * (w["M"] / d["paths"]) if d.get("scale_with_paths", True) else d["bytes"]
    except (OSError, KeyError, ValueError, TypeError):
        return None


def run_gpu(args, w):
    import torch

    import rbergomi_gb300 as R

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    R.lib()
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    prec = R.MIXED if args.precision == "mixed" else R.FP64
    # weak scaling: every rank prices its own M paths (disjoint Philox paths)
    offset = rank * w["M"]
    conv = {"auto": R.CONV_AUTO, "gemm": R.CONV_GEMM, "fft": R.CONV_FFT, "direct": R.CONV_DIRECT}[args.conv]
    kw = dict(seed=w["seed"], precision=prec, split=args.split, path_offset=offset, stream=sptr, conv=conv)
    flush = torch.empty((256 << 20) // 4, dtype=torch.float32, device="cuda")

    # the arguments marshalled once (RtPricer); every step runs the whole call on the device
    pricer = R.RtPricer(w["xi"], w["H"], w["eta"], w["rho"], w["T"], w["K"], w["N"], w["M"], **kw)

    def step():
        return pricer()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    R.profile_reset()
    R.profile_enable(True)
    n0 = R.launch_count()
    times = []
    with ClockSampler(local) as clk:
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            price, stat, iv = step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        price, stat, iv = price.copy(), stat.copy(), iv.copy()  # the pricer reuses its arrays
        if ws > 1:
            torch.distributed.barrier()
    R.profile_enable(False)
    launches = R.launch_count() - n0
    total_ms = float(sum(times))
    if ws > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = ws * path_steps(w) / (ms_step / 1e3)
    if rank != 0:
        return
    stage = R.STAGE_MIXED if prec == R.MIXED else R.STAGE_PATH_FP64
    kms, kn = R.profile_read(stage)
    avg_kernel_ms = kms / max(kn, 1)
    bf16_peak, hbm_peak, peak_src = peaks()
    algo_flops = w["M"] * w["N"] * (w["N"] - 1) * len(set(w["H"])) / max(1, kn // args.steps)
    achieved_tf = algo_flops / (avg_kernel_ms / 1e3) / 1e12
    Np = (w["N"] + 31) // 32 * 32
    nc = Np // 32
    # split products on the tensor pipe: three (16-bit splits) or two (TF32 with one compensation term)
    exec_flops = (4.0 if args.split == 2 else 6.0) * 32 * 32 * nc * (nc + 1) / 2 * w["M"] / max(1, kn // args.steps)
    fp64_fft = args.conv == "fft" or (args.conv == "auto" and 200 <= w["N"] <= 2048)
    kname = ("k_mixed_fft" if (args.conv == "fft" or (args.conv == "auto" and w["N"] > 1024))
             else "k_mixed_gemm") if prec == R.MIXED else ("k_path_fp64_fft" if fp64_fft else "k_path_fp64")
    roof = {"bound": "tensor", "achieved": achieved_tf, "peak": bf16_peak, "unit": "TFLOP/s",
            "frac": achieved_tf / bf16_peak, "traffic": traffic_per_launch(kname, w),
            "kernel": kname,
            "kernel_ms": avg_kernel_ms, "peak_source": f"{peak_src} bf16 burst",
            "algorithmic_flops_per_launch": algo_flops,
            "executed_tensor_tflops": exec_flops / (avg_kernel_ms / 1e3) / 1e12 if prec == R.MIXED else None}

    # plain FP64 form on the same workload, and the error vs FP64 on identical normals
    extra = {}
    if prec == R.MIXED and not args.skip_fp64:
        kf = dict(seed=w["seed"], path_offset=offset, stream=sptr)
        R.price_rt(w["xi"], w["H"], w["eta"], w["rho"], w["T"], w["K"], w["N"], min(w["M"], 1 << 16), **kf)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        R.price_rt(w["xi"], w["H"], w["eta"], w["rho"], w["T"], w["K"], w["N"], w["M"], **kf)
        e1.record(stream)
        torch.cuda.synchronize()
        fp64_ms = e0.elapsed_time(e1)
        fp, fs, _ = R.price_rt(w["xi"], w["H"], w["eta"], w["rho"], w["T"], w["K"], w["N"], w["M"],
                               normals=R.NORMALS_F32, **kf)
        err = np.abs(price - fp)
        extra = {"fp64_value": path_steps(w) / (fp64_ms / 1e3), "fp64_ms_per_step": fp64_ms,
                 "speedup_vs_fp64": (path_steps(w) / (ms_step / 1e3)) / (path_steps(w) / (fp64_ms / 1e3)),
                 "max_rel_err_vs_fp64": float(np.max(err / fp)),
                 "max_err_over_se": float(np.max(err / fs)),
                 "prices": [float(x) for x in price], "stat": [float(x) for x in stat]}

    # e2e through the drop-in C ABI with host buffers
    os.environ["RBG_PRECISION"] = "mixed" if prec == R.MIXED else "fp64"
    seed_words = [w["seed"]]
    for _ in range(max(1, args.warmup // 2)):
        R.computeIVRT_tensor(w["xi"], w["H"], w["eta"], w["rho"], w["T"], w["K"], w["N"], w["M"], seed_words)
    t_e2e = []
    for s in range(args.steps):
        # H moved by a relative 1e-4 per step: every call plans and uploads all of
        # its tables (Gamma strip, compensators, outputs), as a calibration loop
        # with changing parameters does; the work per call is unchanged
        Hs = [h * (1.0 + 1e-4 * (s + 1)) for h in w["H"]]
        t0 = time.perf_counter()
        R.computeIVRT_tensor(w["xi"], Hs, w["eta"], w["rho"], w["T"], w["K"], w["N"], w["M"], seed_words)
        t_e2e.append(time.perf_counter() - t0)
    h2d, d2h = R.last_transfer_bytes()
    e2e = {"value": path_steps(w) / statistics.mean(t_e2e), "unit": "path-steps/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "ms_per_step": 1e3 * statistics.mean(t_e2e), "api": "computeIVRT_tensor (C ABI, host buffers)"}

    cpu = None
    if not args.skip_cpu:
        from oracle import oracle as O
        thr = O.max_threads()
        v, dt = cpu_sample(w, args.cpu_paths, thr)
        cpu = {"value": v, "unit": "path-steps/s", "cores": thr, "kind": "port",
               "sample": f"{args.cpu_paths} paths of this workload, FP64 C restatement, {dt:.1f} s wall"}

    line = {
        "metric": METRIC, "value": value, "unit": "path-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("bf16x3", "f16x3", "tf32x2")[args.split] + "+f32+f64" if prec == R.MIXED else "f64",
        "data": "synthetic (Philox4x32-10 normals generated on device)",
        "config": {"workload": args.workload, "N": w["N"], "M": w["M"], "strikes": len(w["K"]),
                   "H": w["H"], "eta": w["eta"], "rho": w["rho"], "xi": w["xi"], "T": w["T"][0],
                   "seed": w["seed"], "precision": args.precision, "conv": args.conv,
                   "l2": "flushed (256 MiB write) before each step",
                   "prices_per_step": len(w["H"]) * len(w["K"])},
        "prices_per_s": ws * len(w["H"]) * len(w["K"]) / (ms_step / 1e3),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(), "gpu_launches": launches,
    }
    if prec == R.MIXED:
        roof["issue"] = issue_roofline(kname, path_steps(w) / max(1, kn // args.steps), avg_kernel_ms, line["clocks"])
    line.update(extra)
    if ws == 1 and not args.skip_serving:
        # the serving workload (10,000 Poisson requests at 200/s, about a minute),
        # after the timed region of the headline workload
        line["serving"] = serve_stream(args, local)
    print(json.dumps(line))


# ------------------------------------------------------- ParamTot grid arm
GRID_H, GRID_ETA, GRID_RHO = [0.05, 0.1, 0.2, 0.3], [1.0, 1.5, 2.0, 2.5], [-0.95, -0.7, -0.5]
GRID_T = [0.25, 0.5, 1.0, 2.0]
GRID_K = [round(0.7 + 0.06 * i, 10) for i in range(11)]


def run_grid(args):
    """The full ParamTot grid sharing one Gaussian draw: 48 (H, eta, rho) tuples
    (H slowest, rho fastest) x 4 maturities x 11 strikes, 256 steps per unit
    time, M = 2^20, seed 7.  One call per maturity with N_T = 256 T steps:
    the shorter maturities price on prefixes of the same Philox paths.  One
    step = the four calls."""
    import torch

    import rbergomi_gb300 as R

    torch.cuda.set_device(0)
    R.lib()
    stream = torch.cuda.current_stream()
    prec = R.MIXED if args.precision == "mixed" else R.FP64
    M = int(args.paths or (1 << 20))
    H = [h for h in GRID_H for _ in GRID_ETA for _ in GRID_RHO]
    eta = [e for _ in GRID_H for e in GRID_ETA for _ in GRID_RHO]
    rho = [r for _ in GRID_H for _ in GRID_ETA for r in GRID_RHO]
    flush = torch.empty((256 << 20) // 4, dtype=torch.float32, device="cuda")

    def step():
        out = []
        for T in GRID_T:
            out.append(R.price_rt(0.235 ** 2, H, eta, rho, [T] * len(GRID_K), GRID_K, int(256 * T), M, seed=7,
                                  precision=prec, stream=stream.cuda_stream))
        return out

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    n0 = R.launch_count()
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    psteps = M * sum(int(256 * T) for T in GRID_T) * len(GRID_H)
    prices = len(H) * len(GRID_K) * len(GRID_T)
    print(json.dumps({
        "metric": METRIC, "value": psteps / (ms / 1e3), "unit": "path-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == R.FP64 else "bf16x3+f32+f64", "data": "synthetic (Philox4x32-10 normals)",
        "config": {"workload": "paramtot-grid-m1m", "M": M, "tuples": len(H), "maturities": GRID_T,
                   "strikes": len(GRID_K), "steps_per_unit_time": 256, "seed": 7, "precision": args.precision,
                   "l2": "flushed (256 MiB write) before each step"},
        "prices_per_s": prices / (ms / 1e3), "clocks": clk.summary(), "gpu_launches": R.launch_count() - n0,
    }))


def run_sobol(args):
    """Sobol' quasi-Monte Carlo RT pricing, FP64 form (rbg_price_rt_sobol; the
    mixed form on the same points is timed beside it as mixed_value):
    H=0.1, eta=1.9, rho=-0.9, xi=0.235^2, T=1, 21 strikes on [0.6, 1.4], N=256
    (512 Sobol' dimensions), M = 2^20 points.  Direction integers: the
    reference generator's own (rBergomi/sobol.cpp), recovered from its points
    in tests/golden/sobol.npz.  The same call with the Brownian bridge (both
    forms) and the Philox pricers on the same workload are timed beside it."""
    import torch

    import rbergomi_gb300 as R

    torch.cuda.set_device(0)
    R.lib()
    stream = torch.cuda.current_stream()
    V = R.sobol_directions_from_points(np.load(os.path.join(ROOT, "tests", "golden", "sobol.npz"))["gray_points"])
    M, N = int(args.paths or (1 << 20)), int(args.steps_per_path or 256)
    K = list(np.round(np.linspace(0.6, 1.4, 21), 10))
    a = (0.235 ** 2, [0.1], [1.9], [-0.9], [1.0] * 21, K, N, M)
    flush = torch.empty((256 << 20) // 4, dtype=torch.float32, device="cuda")

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        times, out = [], None
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return float(np.mean(times)), out

    n0 = R.launch_count()
    with ClockSampler(0) as clk:
        ms, (pq, sq, _) = timed(lambda: R.price_rt_sobol(*a, V, stream=stream.cuda_stream))
    launches = R.launch_count() - n0
    ms_b, (pb, _, _) = timed(lambda: R.price_rt_sobol(*a, V, bridge=True, stream=stream.cuda_stream))
    ms_p, (pp, sp, _) = timed(lambda: R.price_rt(*a, seed=11, precision=R.FP64, stream=stream.cuda_stream))
    ms_m, (pm, _, _) = timed(lambda: R.price_rt_sobol(*a, V, precision=R.MIXED, stream=stream.cuda_stream))
    ms_pm, _ = timed(lambda: R.price_rt(*a, seed=11, precision=R.MIXED, stream=stream.cuda_stream))
    ms_mb, (pmb, _, _) = timed(lambda: R.price_rt_sobol(*a, V, bridge=True, precision=R.MIXED,
                                                        stream=stream.cuda_stream))
    print(json.dumps({
        "metric": METRIC, "value": M * N / (ms / 1e3), "unit": "path-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "Sobol' points (the reference generator's direction integers)",
        "config": {"workload": "sobol-fp64-n256-m1m", "N": N, "M": M, "strikes": 21, "dims": 2 * N,
                   "l2": "flushed (256 MiB write) before each step"},
        "bridge_value": M * N / (ms_b / 1e3), "philox_fp64_value": M * N / (ms_p / 1e3),
        "mixed_value": M * N / (ms_m / 1e3), "max_rel_diff_mixed_vs_fp64_qmc": float(np.max(np.abs(pm - pq) / pq)),
        "philox_mixed_value": M * N / (ms_pm / 1e3),
        "mixed_bridge_value": M * N / (ms_mb / 1e3),
        "max_rel_diff_mixed_vs_fp64_bridge": float(np.max(np.abs(pmb - pb) / pb)),
        "max_abs_diff_qmc_vs_philox": float(np.max(np.abs(pq - pp))), "philox_stat_max": float(np.max(sp)),
        "max_abs_diff_bridge_vs_plain_qmc": float(np.max(np.abs(pb - pq))),
        "clocks": clk.summary(), "gpu_launches": launches,
    }))


# ------------------------------------------------------------ serving arm
def serving_requests(n: int, rate: float, seed: int = 20261203, small: bool = False):
    """Calibration-style traffic: Poisson arrivals at `rate`/s; H ~ U[.03,.45],
    eta ~ U[.5,3], rho ~ U[-.99,-.3], xi ~ U[.01,.1], T ~ U[.05,3], 1-64 strikes
    on [0.5, 1.5], N and M log-uniform on [64, 1024] and [2^14, 2^22], Philox
    seed = request index.  small: N on [64, 512] and M on [2^14, 2^17] (the
    requests shared launches price), for a saturating stream."""
    n_hi, m_hi = (512, 2 ** 17) if small else (1024, 2 ** 22)
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for i in range(n):
        nk = int(rng.integers(1, 65))
        reqs.append(dict(
            H=[float(rng.uniform(0.03, 0.45))], eta=[float(rng.uniform(0.5, 3.0))], rho=[float(rng.uniform(-0.99, -0.3))],
            xi=float(rng.uniform(0.01, 0.1)), T=[float(rng.uniform(0.05, 3.0))] * nk,
            K=list(np.linspace(0.5, 1.5, nk)) if nk > 1 else [1.0],
            N=int(np.exp(rng.uniform(np.log(64), np.log(n_hi)))),
            M=int(np.exp(rng.uniform(np.log(2 ** 14), np.log(m_hi)))), seed=i, t=float(t[i])))
    return reqs


def serve_stream(args, local: int) -> dict:
    """Replays the Poisson request stream through the serving loop
    (rbg_server_*) and returns its latency, throughput and server figures,
    with the plain FP64 form one request at a time on a sample beside it."""
    import threading

    import rbergomi_gb300 as R

    reqs = serving_requests(args.requests, args.rate, small=args.small_only)
    # warm the kernels and the allocator on a few off-schedule requests
    with R.Server() as srv:
        for r in reqs[:8]:
            srv.wait(srv.submit(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], 1 << 14, seed=r["seed"]))
    lat = np.zeros((len(reqs), 3))
    n0 = R.launch_count()
    with ClockSampler(local) as clk:
        extra = {}
        if args.slots:
            extra["slots"] = args.slots
        if args.high_slots is not None:
            extra["high_priority_slots"] = args.high_slots
        with R.Server(use_graphs=0 if args.no_graphs else 1, batch_wait_us=args.batch_wait_us,
                      batch_slots=args.batch_slots, **extra) as srv:
            tickets = [None] * len(reqs)
            ready = threading.Semaphore(0)

            def submitter():
                t0 = time.perf_counter()
                for i, r in enumerate(reqs):
                    dt = r["t"] - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                    tickets[i] = srv.submit(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], r["M"],
                                            seed=r["seed"])
                    ready.release()

            wall0 = time.perf_counter()
            th = threading.Thread(target=submitter)
            th.start()
            for i in range(len(reqs)):
                ready.acquire()
                lat[i] = srv.wait_timed(tickets[i])[3]
            th.join()
            wall = time.perf_counter() - wall0
            st = srv.stats()
    launches = R.launch_count() - n0
    total = lat[:, 2]
    prices = sum(len(r["K"]) for r in reqs)
    psteps = sum(r["M"] * r["N"] for r in reqs)
    worst = int(np.argmax(total))
    w = reqs[worst]
    # what was in flight when the slowest request arrived: requests submitted in
    # the 50 ms before it that had not finished by its arrival
    t_w = w["t"]
    overlap = [i for i in range(max(0, worst - 200), worst)
               if reqs[i]["t"] + total[i] / 1e3 > t_w]
    # FP64 one-request-at-a-time form on a sample of the same stream
    fp64 = None
    if args.fp64_sample > 0:
        samp = reqs[:args.fp64_sample]
        t0 = time.perf_counter()
        tl = []
        for r in samp:
            t1 = time.perf_counter()
            R.price_rt(r["xi"], r["H"], r["eta"], r["rho"], r["T"], r["K"], r["N"], r["M"], seed=r["seed"])
            tl.append(1e3 * (time.perf_counter() - t1))
        dt = time.perf_counter() - t0
        fp64 = {"requests": len(samp), "prices_per_s": sum(len(r["K"]) for r in samp) / dt,
                "path_steps_per_s": sum(r["M"] * r["N"] for r in samp) / dt,
                "p50_ms_alone": float(np.percentile(tl, 50)), "max_ms_alone": float(np.max(tl)),
                "note": "one request at a time, no queueing: latency is service time only"}
    return {
        "workload": "serving-poisson", "requests": len(reqs), "rate_per_s": args.rate, "graphs": not args.no_graphs,
        "batch_wait_us": args.batch_wait_us, "batch_slots": args.batch_slots, "small_only": args.small_only,
        "slots": args.slots or None, "high_priority_slots": args.high_slots,
        "p50_ms": float(np.percentile(total, 50)), "p99_ms": float(np.percentile(total, 99)),
        "max_ms": float(np.max(total)), "mean_ms": float(np.mean(total)),
        "queue_p99_ms": float(np.percentile(lat[:, 0], 99)), "service_p99_ms": float(np.percentile(lat[:, 1], 99)),
        "prices_per_s": prices / wall, "path_steps_per_s": psteps / wall, "requests_per_s": len(reqs) / wall,
        "wall_s": wall,
        "slowest": {"index": worst, "N": w["N"], "M": w["M"], "strikes": len(w["K"]), "path_steps": w["M"] * w["N"],
                    "queue_ms": float(lat[worst, 0]), "service_ms": float(lat[worst, 1]),
                    "in_flight_at_arrival": len(overlap),
                    "in_flight_path_steps": float(sum(reqs[i]["M"] * reqs[i]["N"] for i in overlap))},
        "server": st, "gpu_launches": launches, "clocks": clk.summary(), "fp64_one_at_a_time": fp64,
    }


def run_serving(args):
    import torch

    import rbergomi_gb300 as R

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    R.lib()
    sv = serve_stream(args, local)
    line = {
        "metric": "serving prices/s (p50/p99 latency ms)", "value": sv["prices_per_s"], "unit": "prices/s",
        "n_gpus": ws, "steps": 1, "warmup": 1, "ms_per_step": 1e3 * sv["wall_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3+f32+f64", "data": "synthetic request stream",
        "config": {"workload": "serving-poisson", "requests": sv["requests"], "rate_per_s": args.rate,
                   "graphs": not args.no_graphs},
        "gpu_launches": sv["gpu_launches"], "clocks": sv["clocks"],
    }
    line.update({k: v for k, v in sv.items() if k not in line})
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT,
                    choices=sorted(WORKLOADS) + ["serving-poisson", "paramtot-grid-m1m", "sobol-fp64-n256-m1m"])
    ap.add_argument("--precision", default=None, choices=["mixed", "fp64"])
    ap.add_argument("--split", type=int, default=0,
                    help="0 = BF16x3, 1 = FP16x3, 2 = TF32 with one compensation term")
    ap.add_argument("--cpu-paths", type=int, default=1 << 18,
                    help="CPU legs: paths per sample (about 20 core-seconds on 16 cores at N = 512)")
    ap.add_argument("--paths", type=int, default=None, help="override M (small cases for ncu captures)")
    ap.add_argument("--steps-per-path", type=int, default=None, help="override N (crossover sweeps)")
    ap.add_argument("--conv", default="auto", choices=["auto", "gemm", "fft", "direct"],
                    help="Volterra backend: gemm / fft (mixed form), fft / direct (FP64 form)")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--requests", type=int, default=10000, help="serving: number of requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: Poisson arrival rate per second")
    ap.add_argument("--fp64-sample", type=int, default=20, help="serving: FP64 one-at-a-time sample size")
    ap.add_argument("--no-graphs", action="store_true", help="serving: launch without CUDA graphs")
    ap.add_argument("--batch-slots", type=int, default=8, help="serving: shared launches in flight (0: none)")
    ap.add_argument("--slots", type=int, default=0, help="serving: request slots (0: the server's default)")
    ap.add_argument("--high-slots", type=int, default=None, help="serving: high-priority request slots")
    ap.add_argument("--small-only", action="store_true",
                    help="serving: only requests shared launches price (N <= 512, M <= 2^17)")
    ap.add_argument("--batch-wait-us", type=float, default=0.0,
                    help="serving: batching window of the shared launches (0: launch what is pending at once)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-serving", action="store_true",
                    help="headline workload: leave out the serving replay that the default line carries")
    args = ap.parse_args()
    if args.workload == "serving-poisson":
        run_serving(args)
        return
    if args.workload == "sobol-fp64-n256-m1m":
        return run_sobol(args)
    if args.workload == "paramtot-grid-m1m":
        args.precision = args.precision or "fp64"
        run_grid(args)
        return
    w = dict(WORKLOADS[args.workload])
    if args.paths:
        w["M"] = int(args.paths)
    if args.steps_per_path:
        w["N"] = int(args.steps_per_path)
    if args.precision is None:
        args.precision = "mixed" if args.workload.startswith("mixed") else "fp64"
    if args.impl == "reference":
        run_reference(args, w)
    else:
        run_gpu(args, w)


if __name__ == "__main__":
    main()
