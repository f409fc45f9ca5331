#!/usr/bin/env python
"""Benchmark: fixed-step RK4 steps/s of the constant-stratification spectral
step (wave-vortex transforms + nonlinear flux + RK4) at 256x256x129.

Workload (one "step" = one WVFixedStepRK4 step = 4 nonlinear fluxes + stage
arithmetic): Lx = Ly = 800 km, Lz = 4000 m, N0 = 5.2e-3 1/s, latitude 33,
nonhydrostatic, 2/3 antialiasing; seeded synthetic state (uniform random
phases, Gaussian amplitudes shaped by (Kh^2 + m^2)^(-3/4), representable via
one inverse/forward round trip, 0.1 m/s rms velocity); dt = 0.5 x the CFL limit.

  value : device-timed RK4 steps/s, state resident in HBM (CUDA events on the
          launching stream, L2 flushed between steps)
  e2e   : the same through the host-pointer C ABI (wv_rk4_steps on the caller's
          pinned arrays), state copied host->device and back every step,
          wall-clock timed
  --impl reference : the reference's own C++ step (WVFixedStepRK4 over its
          CompiledKernel flux, built by oracle/ref_build.sh with the oracle's
          O(N log N) FFT engine) on every host thread, same workload; the numpy
          restatement only where the C++ cannot be built
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "wave-vortex-model_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

GRID = dict(Nx=256, Ny=256, Nz=129, Nj=85, Lx=800e3, Ly=800e3, Lz=4000.0, N0=5.2e-3, latitude=33.0)
METRIC = "RK4 steps/s 256x256x129: mixed vs FP64 plain, same GPU, err<=1e-6; adjoint/fwd"
# The reference's published fixed-step RK4 rate for this grid: standalone C++ with
# FFTW on an 18-thread Apple M5 Max, 2 steps in 0.9078 s (three-interface record).
PUBLISHED_RK4_STEPS_S = 2.20
# The reference's published nonlinearFlux times, compiled C++ with FFTW on the M5 Max
# (core-v1 and three-interface records), ms, keyed (Nx, Nz, hydrostatic).
PUBLISHED_FLUX_MS = {(256, 65, False): 66.68, (256, 65, True): 57.72, (512, 129, False): 526.66,
                     (512, 129, True): 392.81, (256, 129, False): 134.3}
UNIT = "RK4 steps/s"
# how the mixed form's vertical kernels compute (WV_VERTICAL_* names)
_MIXED_VERTICAL = {
    "tensor": "as split-BF16 (3 pieces, 6 products) tcgen05 GEMMs with f32 accumulators",
    "fft": "as f32 FFTs of the even / odd extension over z",
    "cuda": "as the dense folded f32 contraction on the CUDA cores",
}
SEED = 1
URMS = 0.1


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--profile-flux", choices=["fp64", "mixed", "fp32x2"], default=None,
                    help="only run --profile-count nonlinear fluxes of the 256x256x129 workload (for ncu captures)")
    ap.add_argument("--profile-count", type=int, default=3)
    ap.add_argument("--profile-vjp", action="store_true", help="with --profile-flux: also run as many flux VJPs")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="with --profile-flux: one checkpointed RK4 adjoint of 20 steps, checkpoints every 10, instead")
    ap.add_argument("--profile-size", type=int, default=256,
                    help="with --profile-flux: grid N x N x (N/2+1) over 3.125 km x N (256: the benchmark workload)")
    ap.add_argument("--workload", choices=["256", "512"], default="256",
                    help="512: only the 512x512x257 leg (mixed and paired FP32 vs FP64 over --steps-512 RK4 steps)")
    ap.add_argument("--steps-512", type=int, default=200,
                    help="RK4 steps of the 512x512x257 leg (part of the default run; 0 skips it)")
    return ap.parse_args()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))
        return out


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_value(local_seconds, steps, world, dist=None, device="cpu"):
    """Whole-job throughput of `world` replicas that each ran `steps` steps:
    world * steps / (max over ranks of the local time), the max taken with an
    all-reduce (NCCL on the GPU ranks, gloo in the CPU tests)."""
    import torch
    t = float(local_seconds)
    if world > 1 and dist is not None:
        tt = torch.tensor([t], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return world * steps / t, t


def configuration(wvgpu):
    return wvgpu.Configuration(Nx=GRID["Nx"], Ny=GRID["Ny"], Nz=GRID["Nz"], Nj=GRID["Nj"], Lx=GRID["Lx"], Ly=GRID["Ly"],
                               Lz=GRID["Lz"], N0=GRID["N0"], latitude=GRID["latitude"])


def stage_bytes(sizes, nt, s):
    """Algorithmic HBM bytes per launch of each flux stage under this layout
    (s = bytes per complex of the xy working type), as in the design notes:
      vertical inverse: read Ap,Am,A0 (+omega) and write (4+nt) z-grid channels of the active rows
      y inverse:        read (4+nt) channels of active rows, write (4+2nt) channels x Ny x kx columns
      x products:       read (4+2nt) channels x Ny x kx, write nt channels x Ny x kx
      y forward:        read nt x Ny x kx, write nt channels of the active rows
      vertical forward: read nt channels of active rows and Ap,Am,A0 (+omega), write Fp,Fm,F0"""
    M, P, KX = sizes["M"], sizes["active_rows"], sizes["kx_columns"]
    Ny, Nz = GRID["Ny"], GRID["Nz"]
    col = Nz * P * s
    grid = Nz * Ny * KX * s
    return {
        "vertical_inverse": 3 * 16 * M + 8 * M + (4 + nt) * col,
        "y_inverse": (4 + nt) * col + (4 + 2 * nt) * grid,
        "x_products": (4 + 2 * nt) * grid + nt * grid,
        "y_forward": nt * grid + nt * col,
        "vertical_forward": nt * col + 3 * 16 * M + 8 * M + 3 * 16 * M,
    }


def fp64_peak_tflops(torch):
    """FP64 throughput of this GPU, measured with a float64 GEMM (cuBLAS)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def traffic_from_profile(stage, precision="fp64"):
    """Per-launch DRAM bytes of a stage from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) >= 3 and not line.startswith("#") and parts[0] == stage and parts[1] == precision:
                return float(parts[2])
    return None


REF_WORKLOAD_CASE = dict(Nx=GRID["Nx"], Ny=GRID["Ny"], Nz=GRID["Nz"], Nj=GRID["Nj"], Lx=GRID["Lx"], Ly=GRID["Ly"],
                         Lz=GRID["Lz"], latitude=GRID["latitude"], isHydrostatic=False, shouldAntialias=True,
                         damping=False)


def _reference_cpp():
    """The reference's own C++ (CompiledKernel + PortableRuntime fixed-step RK4,
    built by oracle/ref_build.sh on this host) with the oracle's O(N log N) FFT
    engine; None when it cannot be built here."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_lib as R
    if not R.available():
        return None
    return R


def _host_cpu():
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def reference_cpp_steps(state, dt, steps, warmup, budget_s):
    """WVFixedStepRK4::step of the reference's C++ on the 256x256x129 state:
    (seconds per step, steps timed, threads, sample text), or None."""
    R = _reference_cpp()
    if R is None:
        return None
    lib = R.load_lib()
    ref = R.Ref(lib, REF_WORKLOAD_CASE, R.ENGINE_ORACLE_FFT)
    Ap, Am, A0 = state
    t = 0.0
    for _ in range(warmup):
        Ap, Am, A0, t = ref.rk4(Ap, Am, A0, t, 0.0, dt, 1)
    done, el = 0, 0.0
    w0 = time.perf_counter()
    while done < steps:
        Ap, Am, A0, t = ref.rk4(Ap, Am, A0, t, 0.0, dt, 1)
        done += 1
        el = time.perf_counter() - w0
        if el > budget_s:
            break
    threads = int(lib.wvref_oracle_fft_threads())
    sample = (f"{done} WVFixedStepRK4 steps (4 nonlinear fluxes each) of the 256x256x129 state after {warmup} warm-up "
              f"step(s): the reference's own C++ (CompiledKernel + PortableRuntime, -O3, 2 coefficient workers as "
              f"published) with the oracle's O(N log N) FFT engine on {threads} threads standing in for FFTW "
              f"(absent here); host {_host_cpu()}, {os.cpu_count()} cores")
    return el / done, done, threads, sample, (Ap, Am, A0, t, warmup + done)


def cpu_baseline(state, dt):
    """Bounded CPU sample of the same workload: 2 RK4 steps of the reference's
    own C++ (1 warm-up), else 1 step of the numpy restatement."""
    r = reference_cpp_steps(state, dt, steps=2, warmup=1, budget_s=60.0)
    if r is not None:
        per, done, threads, sample, final = r
        return {"value": 1.0 / per, "unit": UNIT, "cores": threads, "kind": "reference", "sample": sample}, final
    return cpu_baseline_oracle(state, dt), None


def cpu_baseline_oracle(state, dt):
    """One RK4 step of the CPU oracle (numpy/scipy restatement of the reference)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import wv_oracle as O
    c = O.Config(Nx=GRID["Nx"], Ny=GRID["Ny"], Nz=GRID["Nz"], Nj=GRID["Nj"], Lx=GRID["Lx"], Ly=GRID["Ly"], Lz=GRID["Lz"],
                 N0=GRID["N0"], latitude=GRID["latitude"])
    d = O.build_descriptor(c)
    Ap, Am, A0 = state
    O.rk4_step(d, Ap, Am, A0, 0.0, 0.0, dt)  # warm (FFT plans, page-in)
    t = time.perf_counter()
    O.rk4_step(d, Ap, Am, A0, 0.0, 0.0, dt)
    el = time.perf_counter() - t
    return {"value": 1.0 / el, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "1 RK4 step (4 nonlinear fluxes) of the 256x256x129 state with the numpy/scipy oracle "
                      "(scipy.fft workers=-1); seconds per step %.2f" % el}


def _time_steps(k, dev, t, t0, dt, steps, warmup, stream, barrier, flush, torch):
    """Device time (ms) of `steps` RK4 steps, one event pair per step, L2 flushed between."""
    for _ in range(warmup):
        _, _, _, t = k.rk4(*dev, t, t0, dt, 1)
    barrier()
    total = 0.0
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, _, _, t = k.rk4(*dev, t, t0, dt, 1)
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    barrier()
    return total, t


def _stage_profile(k, dev, t, t0, dt, precision, torch):
    k.setStageInstrumentation(True)
    k.rk4(*dev, t, t0, dt, 1)
    torch.cuda.synchronize()
    st = k.stage_times()
    k.setStageInstrumentation(False)
    names = ["vertical_inverse", "y_inverse", "x_products", "y_forward", "vertical_forward"]
    per_launch = {n: st[n + "_ms"] / max(st["fluxes"], 1) for n in names}
    dominant = max(per_launch, key=per_launch.get)
    s = 8 if precision == "mixed" else 16  # bytes per complex of the working type (paired FP32: 16)
    sbytes = stage_bytes(k.sizes, 4, s)
    peaks, peak_kind = measured_peaks()
    achieved = sbytes[dominant] / (per_launch[dominant] * 1e-3) / 1e9
    flux_ms = sum(per_launch.values())
    M, P = k.sizes["M"], k.sizes["active_rows"]
    b_flux = 104 * M + 24 * s * P * GRID["Nz"]
    # arithmetic of the x pass (the dominant stage): per (y, z) row, 15 inverse and 4
    # forward real transforms as complex lines of L = Nx/2 (5 L log2 L flops per line
    # plus ~10 flops per entry for the real-transform pre/post twiddles) and the
    # products (6 flops per point and target)
    import math
    L = GRID["Nx"] // 2
    rows = GRID["Ny"] * GRID["Nz"]
    x_flops = rows * (19 * (5 * L * math.log2(L) + 10 * L) + 4 * GRID["Nx"] * 6)
    x_ms = per_launch["x_products"]
    compute = {"stage": "x_products", "flops_per_launch": x_flops, "achieved_tflops": x_flops / (x_ms * 1e-3) / 1e12,
               "pipe": "fp64" if precision == "fp64" else "fp32"}
    return {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "compute": compute,
            "frac": achieved / peaks["hbm_gbs"], "traffic": traffic_from_profile(dominant, precision),
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum per launch from a committed ncu capture "
                              "of this kernel on this workload (profiles/ncu_traffic.txt), not from this run",
            "peak_source": peak_kind, "algorithmic_bytes_per_launch": sbytes[dominant],
            "avg_launch_ms": per_launch[dominant], "stage_ms_per_flux": per_launch,
            "flux": {"algorithmic_bytes": b_flux, "ms": flux_ms, "achieved_gbs": b_flux / (flux_ms * 1e-3) / 1e9,
                     "frac": b_flux / (flux_ms * 1e-3) / 1e9 / peaks["hbm_gbs"]}}


_FP64_FIELDS = {}


def _field_error_after(kd, km, state, dt, steps, torch, np):
    """Relative L2 error per field (u, v, w, eta) of a reduced-precision handle
    against FP64 after `steps` RK4 steps (the FP64 run is made once per state)."""
    key = (id(kd), steps, dt)
    if key not in _FP64_FIELDS:
        d64 = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
        _, _, _, t1 = kd.rk4(*d64, 0.0, 0.0, dt, steps)
        torch.cuda.synchronize()
        _FP64_FIELDS[key] = (t1, kd.transformWaveVortexToUVWEta(t1, 0.0, *(x.cpu().numpy() for x in d64)))
    t1, f64 = _FP64_FIELDS[key]
    d32 = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
    km.rk4(*d32, 0.0, 0.0, dt, steps)
    torch.cuda.synchronize()
    f32 = kd.transformWaveVortexToUVWEta(t1, 0.0, *(x.cpu().numpy() for x in d32))
    return [float(np.linalg.norm(f32[i] - f64[i]) / np.linalg.norm(f64[i])) for i in range(4)]


def _published_flux_comparison(wvgpu, torch, np):
    """nonlinearFlux device time at the grids the reference publishes flux times
    for (15 km x 15 km x 1.3 km, the published records' domain; seeded spectrum
    state), per precision, beside the published CPU milliseconds."""
    out = []
    for (N, Nz, hydro), ms_ref in PUBLISHED_FLUX_MS.items():
        cfg = wvgpu.Configuration(Nx=N, Ny=N, Nz=Nz, Nj=(2 * (Nz - 1)) // 3, Lx=15e3, Ly=15e3, Lz=1300.0,
                                  latitude=33.0, isHydrostatic=hydro)
        row = {"grid": [N, N, Nz], "hydrostatic": hydro, "published_cpu_ms": ms_ref}
        k64 = wvgpu.WVTransformConstantStratificationKernel(cfg, precision="fp64")
        state = wvgpu.synthetic_state(k64, seed=SEED, urms=URMS)
        dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
        for prec in ("fp64", "fp32x2", "mixed"):
            k = k64 if prec == "fp64" else wvgpu.WVTransformConstantStratificationKernel(cfg, precision=prec)
            res = tuple(torch.empty_like(dev[0]) for _ in range(3))
            for _ in range(2):
                k.nonlinearFlux(0.0, 0.0, *dev, out=res)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(5):
                k.nonlinearFlux(0.0, 0.0, *dev, out=res)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1) / 5
            row[prec + "_ms"] = ms
            row[prec + "_speedup_vs_published"] = ms_ref / ms
            if k is not k64:
                k.close()
        k64.close()
        out.append(row)
    return out


def _adjoint_timing(wvgpu, precision, stream, torch, np, repeats=2):
    """Gradient of a final-state misfit through 50 RK4 steps at 128x128x65
    (400 km x 400 km x 4 km), checkpoints every 10 steps: device time of the
    forward run against the checkpointed adjoint (forward pass with
    checkpoints, per-segment recompute, backward sweep)."""
    Nx, Ny, Nz, steps, K = 128, 128, 65, 50, 10
    cfg = wvgpu.Configuration(Nx=Nx, Ny=Ny, Nz=Nz, Nj=(2 * (Nz - 1)) // 3, Lx=400e3, Ly=400e3, Lz=4000.0, latitude=33.0)
    k = wvgpu.WVTransformConstantStratificationKernel(cfg, precision=precision)
    state = wvgpu.synthetic_state(k, seed=SEED, urms=URMS)
    dt = wvgpu.cfl_time_step(k, *state)
    dev0 = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
    # misfit cotangent (u, v, eta)(T) - target at a representative size; its value does not change the cost
    target = wvgpu.synthetic_state(k, seed=SEED + 1, urms=URMS)
    misfit = (k.transformWaveVortexToUVWEta(0.0, 0.0, *state) - k.transformWaveVortexToUVWEta(0.0, 0.0, *target))
    misfit[2] = 0.0
    yb = k.inverse_vjp(steps * dt, 0.0, torch.from_numpy(np.ascontiguousarray(misfit)).cuda())

    def timed(fn):
        best = float("inf")
        for r in range(repeats + 1):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            if r > 0:
                best = min(best, e0.elapsed_time(e1))
        return best

    fwd_ms = timed(lambda: k.rk4(*[x.clone() for x in dev0], 0.0, 0.0, dt, steps))
    adj_ms = timed(lambda: k.rk4_adjoint(*dev0, 0.0, 0.0, dt, steps, K, *yb))
    out = {"grid": [Nx, Ny, Nz], "steps": steps, "checkpoint_every": K, "dt_s": dt, "forward_ms": fwd_ms,
           "adjoint_ms": adj_ms, "adjoint_over_forward": adj_ms / fwd_ms,
           "device_bytes": k.metrics()["device_bytes"]}
    k.close()
    return out


ENSEMBLE_GROUPS = [(64, 33), (128, 65), (192, 97)]
ENSEMBLE_MEMBERS = 32


def _ensemble_timing(wvgpu, stream, torch, np, steps=100, single_steps=20):
    """96-member ensemble of uneven grids (32 each of 64x64x33, 128x128x65,
    192x192x97; 3.125 km per grid point, Lz = 4 km), mixed precision.  Members
    seeded independently from the bench spectrum at 0.05-0.2 m/s rms; each
    group steps at the smallest CFL step of its members.  The ensemble's
    `steps`-step integration is one CUDA-graph launch; the same members stepped
    one at a time through single-state handles give the comparison rate."""
    cfgs, singles, X, dts = [], [], [], []
    seed = 1000
    for Nx, Nz in ENSEMBLE_GROUPS:
        cfg = wvgpu.Configuration(Nx=Nx, Ny=Nx, Nz=Nz, Nj=(2 * (Nz - 1)) // 3, Lx=3125.0 * Nx, Ly=3125.0 * Nx,
                                  Lz=4000.0, latitude=33.0)
        k = wvgpu.WVTransformConstantStratificationKernel(cfg, precision="mixed")
        states, dd = [], []
        for m in range(ENSEMBLE_MEMBERS):
            A = wvgpu.synthetic_state(k, seed=seed, urms=0.05 + 0.15 * m / (ENSEMBLE_MEMBERS - 1))
            seed += 1
            dd.append(wvgpu.cfl_time_step(k, *A))
            states.append(np.stack(A))
        cfgs.append(cfg)
        singles.append(k)
        X.append(torch.from_numpy(np.ascontiguousarray(np.stack(states))).cuda())
        dts.append(min(dd))
    w0 = time.perf_counter()
    ens = wvgpu.WVEnsemble(cfgs, [ENSEMBLE_MEMBERS] * len(cfgs), precision="mixed", autotune=True)
    create_s = time.perf_counter() - w0
    work = [x.clone() for x in X]
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    ens.rk4(work, 0.0, 0.0, dts, steps)  # capture + instantiate + first run
    torch.cuda.synchronize()
    first_s = time.perf_counter() - w0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ens.rk4(work, 0.0, 0.0, dts, steps)  # same key: replay of the instantiated graph
    e1.record(stream)
    e1.synchronize()
    graph_ms = e0.elapsed_time(e1)
    member_steps = steps * ENSEMBLE_MEMBERS * len(cfgs)
    # the same members one at a time, single-state handles; one untimed step per
    # handle first, so that its first-call set-up stays outside the timed region
    # as the graph's capture does
    for k, x, dt in zip(singles, X, dts):
        w = x[0].clone()
        k.rk4(w[0], w[1], w[2], 0.0, 0.0, dt, 1)
    single = [x.clone() for x in X]
    torch.cuda.synchronize()
    e0.record(stream)
    for k, x, dt in zip(singles, single, dts):
        for m in range(ENSEMBLE_MEMBERS):
            k.rk4(x[m, 0], x[m, 1], x[m, 2], 0.0, 0.0, dt, single_steps)
    e1.record(stream)
    e1.synchronize()
    single_ms = e0.elapsed_time(e1)
    single_rate = single_steps * ENSEMBLE_MEMBERS * len(cfgs) / (single_ms * 1e-3)
    out = {"members": [[Nx, Nx, Nz, ENSEMBLE_MEMBERS] for Nx, Nz in ENSEMBLE_GROUPS], "precision": "mixed",
           "steps": steps, "dt_s": dts, "graph_launches_per_call": 1,
           "value": member_steps / (graph_ms * 1e-3), "unit": "member RK4 steps/s", "ms": graph_ms,
           "one_at_a_time": {"value": single_rate, "unit": "member RK4 steps/s", "steps": single_steps,
                             "ms": single_ms},
           "speedup_vs_one_at_a_time": member_steps / (graph_ms * 1e-3) / single_rate,
           "first_call_s_with_capture": first_s, "create_s_with_autotune": create_s,
           "tuning": ens.tuning(), "metrics": ens.metrics()}
    ens.close()
    for k in singles:
        k.close()
    return out


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    world, rank, local = dist_setup()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import wvgpu
    from wvgpu import build
    build.build()
    cfg = configuration(wvgpu)
    k = wvgpu.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    state = wvgpu.synthetic_state(k, seed=SEED, urms=URMS)
    dt = wvgpu.cfl_time_step(k, *state)
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        return replica_value(x, 1, 1 if world == 1 else world, dist if world > 1 else None, "cuda")[1]

    t0 = 0.0
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
    launches0 = k.metrics()["kernel_launches"]
    with ClockSampler(local) as clocks:
        total_ms, t = _time_steps(k, dev, 0.0, t0, dt, args.steps, args.warmup, stream, barrier, flush, torch)
    # every step launches the same kernels: the timed steps' share of the count
    launches = (k.metrics()["kernel_launches"] - launches0) * args.steps // (args.steps + args.warmup)
    t_s = max_over_ranks(total_ms / 1e3)
    value = world * args.steps / t_s
    roofline = _stage_profile(k, dev, t, t0, dt, "fp64", torch)
    try:
        roofline["fp64_gemm_peak_tflops_measured"] = fp64_peak_tflops(torch)
        roofline["compute"]["frac_of_fp64_gemm_peak"] = (roofline["compute"]["achieved_tflops"] /
                                                         roofline["fp64_gemm_peak_tflops_measured"])
    except Exception:  # pragma: no cover
        roofline["fp64_gemm_peak_tflops_measured"] = None

    # mixed-precision form on the same state
    km = wvgpu.WVTransformConstantStratificationKernel(cfg, precision="mixed")
    devm = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
    mixed_ms, tm = _time_steps(km, devm, 0.0, t0, dt, args.steps, args.warmup, stream, barrier, flush, torch)
    mixed_value = world * args.steps / max_over_ranks(mixed_ms / 1e3)
    vk = km.vertical_kernels()
    mixed = {"value": mixed_value, "unit": UNIT, "ms_per_step": mixed_ms / args.steps,
             "speedup_vs_fp64": mixed_value / value,
             "dtype": "f32 xy transforms and products; vertical inverse " + _MIXED_VERTICAL[vk[0]] + "; vertical forward "
                      + _MIXED_VERTICAL[vk[1]] + "; f32 projection; f64 phase angles and RK4",
             "vertical_kernel": {"inverse": vk[0], "forward": vk[1]},
             "roofline": _stage_profile(km, devm, tm, t0, dt, "mixed", torch)}
    if rank == 0:
        mixed["rel_field_err_vs_fp64_after_100_steps"] = _field_error_after(k, km, state, dt, 100, torch, np)
    mixed["device_status"] = km.device_status()
    # the same with both vertical transforms on the tensor cores (split-BF16 GEMMs), and
    # with both as dense contractions on the CUDA cores
    for name, kind in (("tensor_core_vertical", "tensor"), ("cuda_core_vertical", "cuda")):
        km.set_vertical_kernel(kind)
        v_ms, tm = _time_steps(km, devm, tm, t0, dt, args.steps, args.warmup, stream, barrier, flush, torch)
        v_value = world * args.steps / max_over_ranks(v_ms / 1e3)
        mixed[name] = {
            "value": v_value, "unit": UNIT, "ms_per_step": v_ms / args.steps, "speedup_vs_fp64": v_value / value,
            "stage_ms_per_flux": _stage_profile(km, devm, tm, t0, dt, "mixed", torch)["stage_ms_per_flux"]}
        if rank == 0:
            mixed[name]["rel_field_err_vs_fp64_after_100_steps"] = _field_error_after(k, km, state, dt, 100, torch, np)
    km.close()
    # paired-FP32 form (FP32X2): FP64-class accuracy on the FP32 pipe
    kx = wvgpu.WVTransformConstantStratificationKernel(cfg, precision="fp32x2")
    devx = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
    x_ms, tx = _time_steps(kx, devx, 0.0, t0, dt, args.steps, args.warmup, stream, barrier, flush, torch)
    x_value = world * args.steps / max_over_ranks(x_ms / 1e3)
    fp32x2 = {"value": x_value, "unit": UNIT, "ms_per_step": x_ms / args.steps, "speedup_vs_fp64": x_value / value,
              "dtype": "paired f32 (float-float, ~45-48 significand bits on the FP32 pipe) for the xy transforms, "
                       "products, phases and the vertical transforms (FFTs of the even / odd extension over z); "
                       "f64 angles, stores and RK4",
              "vertical_kernel": kx.vertical_kernel(),
              "roofline": _stage_profile(kx, devx, tx, t0, dt, "fp32x2", torch)}
    if rank == 0:
        err = _field_error_after(k, kx, state, dt, 100, torch, np)
        fp32x2["rel_field_err_vs_fp64_after_100_steps"] = err
        fp32x2["meets_target_3x_and_1e-6"] = bool(fp32x2["speedup_vs_fp64"] >= 3.0 and max(err) <= 1e-6)
    kx.close()
    adjoint = ({p: _adjoint_timing(wvgpu, p, stream, torch, np) for p in ("fp64", "mixed", "fp32x2")}
               if rank == 0 else None)
    ensemble = _ensemble_timing(wvgpu, stream, torch, np) if rank == 0 and not args.no_ensemble else None
    published = _published_flux_comparison(wvgpu, torch, np) if rank == 0 else None

    # end to end through the host-pointer C ABI (wv_rk4_steps, the call the
    # reference's C++ / MEX callers make): the caller's pinned host arrays are
    # copied to the device, stepped and copied back in place on every call
    host = [torch.empty(a.shape, dtype=torch.complex128, pin_memory=True).numpy() for a in state]
    for hbuf, a in zip(host, state):
        hbuf[...] = a
    import ctypes
    lib = wvgpu.load_library()
    te = ctypes.c_double(0.0)

    def host_step():
        rc = lib.wv_rk4_steps(k._h, host[0].ctypes.data, host[1].ctypes.data, host[2].ctypes.data, ctypes.byref(te),
                              float(t0), float(dt), 1)
        if rc != 0:
            raise RuntimeError(lib.wv_last_message(k._h).decode())

    host_step()  # warm the host path
    barrier()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e2e_s = max_over_ranks(time.perf_counter() - w0)
    M = k.sizes["M"]
    coeff_bytes = 3 * M * 16
    g512 = _leg_512(wvgpu, stream, torch, np, args.steps_512) if rank == 0 and args.steps_512 > 0 else None
    cpu, vs_ref = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, final = cpu_baseline(state, dt)
        if final is not None:
            vs_ref = _error_vs_reference_cpp(wvgpu, cfg, k, state, dt, final, torch, np)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / PUBLISHED_RK4_STEPS_S,
        "vs_baseline_source": "published fixed-step RK4 at 256x256x129, standalone C++ (FFTW) on an 18-thread Apple "
                              "M5 Max: 2.20 steps/s (the reference's three-interface record; its run includes an "
                              "observer graph)",
        "dtype": "f64", "data": "synthetic",
        "precision": "fp64 (plain drop-in); the reduced-precision forms are reported under 'mixed' (f32; its "
                     "split-BF16 tensor-core vertical transforms under mixed.tensor_core_vertical) and 'fp32x2' "
                     "(paired f32)",
        "vertical_kernel": k.vertical_kernel(),
        "config": {
            "workload": "fixed-step RK4, nonlinear advection, 256x256x129, 800 km x 800 km x 4 km, N0 5.2e-3, lat 33, "
                        "0.1 m/s rms seeded spectrum state, dt = 0.5 x CFL",
            "grid": [GRID["Nx"], GRID["Ny"], GRID["Nz"]], "Nj": GRID["Nj"], "Nkl": k.sizes["Nkl"], "dt_s": dt,
            "parallelism": f"replicas x{world}", "l2": "flushed between timed steps (256 MB write)"},
        "e2e": {"value": world * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": coeff_bytes,
                "d2h_bytes_per_step": coeff_bytes},
        "gpu_launches": launches,
        "roofline": roofline,
        "mixed": mixed,
        "fp32x2": fp32x2,
        "adjoint": adjoint,
        "ensemble": ensemble,
        "published_flux_comparison": published,
        "grid_512x512x257": g512,
        "error_vs_reference_cpp": vs_ref,
        "clocks": clocks.summary(),
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if rank == 0:
        out["summary"] = _summary(value, mixed, fp32x2, adjoint, ensemble, g512, vs_ref, roofline)
        print(json.dumps(out), flush=True)
    k.close()
    if world > 1:
        dist.destroy_process_group()


def _error_vs_reference_cpp(wvgpu, cfg, k64, state, dt, final, torch, np):
    """Each precision against the reference's own C++ FP64 (WVFixedStepRK4, the
    oracle FFT engine): relative L2 error per field (u, v, w, eta) after the same
    RK4 steps from the same state, and max |F - F_ref| / max |F_ref| of the flux
    at the initial state."""
    R = _reference_cpp()
    Rp, Rm, R0, tr, nsteps = final
    ref_fields = k64.transformWaveVortexToUVWEta(tr, 0.0, Rp, Rm, R0)
    ref = R.Ref(R.load_lib(), REF_WORKLOAD_CASE, R.ENGINE_ORACLE_FFT)
    ref_flux = ref.flux(*state, 0.0, 0.0)
    del ref
    out = {"steps": nsteps, "norm": "field: ||f - f_ref||_2 / ||f_ref||_2 per (u, v, w, eta); "
                                    "flux: max|F - F_ref| / max|F_ref| per (Fp, Fm, F0)"}
    for prec in ("fp64", "fp32x2", "mixed"):
        kk = k64 if prec == "fp64" else wvgpu.WVTransformConstantStratificationKernel(cfg, precision=prec)
        dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
        F = kk.nonlinearFlux(0.0, 0.0, *dev)
        _, _, _, t1 = kk.rk4(*dev, 0.0, 0.0, dt, nsteps)
        torch.cuda.synchronize()
        f = k64.transformWaveVortexToUVWEta(t1, 0.0, *(x.cpu().numpy() for x in dev))
        out[prec] = {
            "rel_field_err": [float(np.linalg.norm(f[i] - ref_fields[i]) / np.linalg.norm(ref_fields[i])) for i in range(4)],
            "rel_flux_err": [float(np.max(np.abs(a.cpu().numpy() - b)) / np.max(np.abs(b))) for a, b in zip(F, ref_flux)]}
        if kk is not k64:
            kk.close()
    return out


def _summary(value, mixed, fp32x2, adjoint, ensemble, g512, vs_ref, roofline):
    """The metric's own figures as flat scalars, last on the line."""
    ok = [(f, d) for f, d in (("fp32x2", fp32x2), ("mixed", mixed))
          if d and max(d.get("rel_field_err_vs_fp64_after_100_steps", [1.0])) <= 1e-6]
    best = max(ok, key=lambda fd: fd[1]["value"]) if ok else None
    s = {"fp64_steps_s": value,
         "form_meeting_1e-6": best[0] if best else None,
         "speedup_at_1e-6_vs_fp64": best[1]["speedup_vs_fp64"] if best else None,
         "fp32x2_speedup_vs_fp64": fp32x2["speedup_vs_fp64"],
         "fp32x2_max_field_err_100": max(fp32x2.get("rel_field_err_vs_fp64_after_100_steps", [float("nan")])),
         "mixed_speedup_vs_fp64": mixed["speedup_vs_fp64"],
         "mixed_field_err_100": mixed.get("rel_field_err_vs_fp64_after_100_steps"),
         "mixed_all_tensor_core_vertical_speedup_vs_fp64": mixed.get("tensor_core_vertical", {}).get("speedup_vs_fp64"),
         "flux_hbm_frac_mixed": mixed["roofline"]["flux"]["frac"],
         "flux_hbm_frac_fp64": roofline["flux"]["frac"]}
    if adjoint:
        for p, a in adjoint.items():
            s[f"adjoint_over_forward_{p}"] = a["adjoint_over_forward"]
    if ensemble:
        s["ensemble_speedup_vs_one_at_a_time"] = ensemble["speedup_vs_one_at_a_time"]
    if g512:
        s["g512_fp64_steps_s"] = g512["fp64"]["value"]
        for p in ("fp32x2", "mixed"):
            s[f"g512_{p}_speedup_vs_fp64"] = g512[p]["speedup_vs_fp64"]
            s[f"g512_{p}_max_field_err_{g512['steps']}"] = max(g512[p]["rel_field_err_vs_fp64"])
    if vs_ref:
        for p in ("fp64", "fp32x2", "mixed"):
            s[f"{p}_max_field_err_vs_reference_cpp_{vs_ref['steps']}_steps"] = max(vs_ref[p]["rel_field_err"])
    return s


def run_reference(args):
    """The reference arm: the reference's own CPU implementation of the step on
    this host's cores -- its C++ CompiledKernel + PortableRuntime WVFixedStepRK4
    (oracle/ref_build.sh; the oracle's O(N log N) FFT engine in place of FFTW) --
    on the same 256x256x129 state and dt.  Falls back to the numpy restatement
    only when the C++ cannot be built on this host.  Rank 0 alone runs."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import wv_oracle as O
    c = O.Config(Nx=GRID["Nx"], Ny=GRID["Ny"], Nz=GRID["Nz"], Nj=GRID["Nj"], Lx=GRID["Lx"], Ly=GRID["Ly"], Lz=GRID["Lz"],
                 N0=GRID["N0"], latitude=GRID["latitude"])
    d = O.build_descriptor(c)
    Ap, Am, A0 = O.spectrum_state(d, seed=SEED, urms=URMS)
    dt = O.cfl_time_step(d, Ap, Am, A0)
    budget = 150.0
    warm = min(args.warmup, 1)
    r = reference_cpp_steps((Ap, Am, A0), dt, args.steps, warm, budget)
    if r is not None:
        per, done, threads, sample, _ = r
        kind, cores = "reference", threads
        sample += f"; {done} of {args.steps} requested steps, capped at {budget:.0f} s"
    else:
        t, t0 = 0.0, 0.0
        for _ in range(warm):
            Ap, Am, A0, t = O.rk4_step(d, Ap, Am, A0, t, t0, dt)
        done, el = 0, 0.0
        w0 = time.perf_counter()
        while done < args.steps:
            Ap, Am, A0, t = O.rk4_step(d, Ap, Am, A0, t, t0, dt)
            done += 1
            el = time.perf_counter() - w0
            if el > budget:
                break
        per = el / done
        kind, cores = "port", os.cpu_count()
        sample = (f"{done} of {args.steps} RK4 steps of the 256x256x129 state (4 nonlinear fluxes each) with the "
                  f"numpy/scipy restatement of the reference kernel (the reference's C++ could not be built here), "
                  f"{warm} warm-up step; capped at {budget:.0f} s")
    value = 1.0 / per
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * per, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": value / PUBLISHED_RK4_STEPS_S, "dtype": "f64",
           "data": "synthetic", "impl": "reference",
           "config": {"workload": "fixed-step RK4, nonlinear advection, 256x256x129, 800 km x 800 km x 4 km, N0 5.2e-3, "
                                  "lat 33, 0.1 m/s rms seeded spectrum state, dt = 0.5 x CFL",
                      "grid": [GRID["Nx"], GRID["Ny"], GRID["Nz"]], "Nj": GRID["Nj"], "Nkl": d.Nkl, "dt_s": dt,
                      "parallelism": "host threads", "l2": "not applicable (CPU arm)"},
           "steps_timed": done, "precision": "fp64",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def _energy(k, state, t, t0, np):
    """0.5 <u^2 + v^2 + w^2 + N0^2 eta^2> over the grid (trapezoid weights in z):
    a physical-space energy diagnostic for drift."""
    f = k.transformWaveVortexToUVWEta(t, t0, *state)
    wz = np.ones(f.shape[1])
    wz[0] = wz[-1] = 0.5
    N0 = k.configuration.N0
    e = f[0] ** 2 + f[1] ** 2 + f[2] ** 2 + (N0 * f[3]) ** 2
    return 0.5 * float(np.sum(e * wz[:, None, None]) / (np.sum(wz) * f.shape[2] * f.shape[3]))


def _leg_512(wvgpu, stream, torch, np, steps):
    """512x512x257 over the 800 km x 800 km x 4 km domain of the 256 workload, seeded
    spectrum state at 0.1 m/s (seed 2), dt = 0.5 CFL: RK4 steps/s of the FP64, mixed
    and paired-FP32 forms over `steps` steps, per-field relative L2 error of the
    reduced forms against FP64 after the run, and the energy drift of each."""
    cfg = wvgpu.Configuration(Nx=512, Ny=512, Nz=257, Nj=170, Lx=800e3, Ly=800e3, Lz=4000.0, N0=5.2e-3, latitude=33.0)
    k = wvgpu.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    state = wvgpu.synthetic_state(k, seed=2, urms=URMS)
    dt = wvgpu.cfl_time_step(k, *state)
    out = {"workload": "512x512x257, 800 km x 800 km x 4 km, N0 5.2e-3, lat 33, 0.1 m/s rms seeded spectrum (seed 2), "
                       "dt = 0.5 x CFL", "steps": steps, "dt_s": dt, "unit": UNIT}
    E0 = _energy(k, state, 0.0, 0.0, np)
    finals = {}
    for name in ("fp64", "mixed", "fp32x2"):
        kk = k if name == "fp64" else wvgpu.WVTransformConstantStratificationKernel(cfg, precision=name)
        dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
        kk.rk4(*[x.clone() for x in dev], 0.0, 0.0, dt, 2)  # warm
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, _, _, tT = kk.rk4(*dev, 0.0, 0.0, dt, steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        finals[name] = [x.cpu().numpy() for x in dev]
        vk = kk.vertical_kernels()
        out[name] = {"value": steps / (ms * 1e-3), "ms_per_step": ms / steps,
                     "vertical_kernel": {"inverse": vk[0], "forward": vk[1]},
                     "energy_drift": (_energy(k, finals[name], tT, 0.0, np) - E0) / E0}
        if kk is not k:
            kk.close()
        del dev
    f64 = k.transformWaveVortexToUVWEta(tT, 0.0, *finals["fp64"])
    for name in ("mixed", "fp32x2"):
        fr = k.transformWaveVortexToUVWEta(tT, 0.0, *finals[name])
        out[name]["rel_field_err_vs_fp64"] = [float(np.linalg.norm(fr[i] - f64[i]) / np.linalg.norm(f64[i]))
                                              for i in range(4)]
        out[name]["speedup_vs_fp64"] = out[name]["value"] / out["fp64"]["value"]
    k.close()
    return out


def run_workload_512(args):
    """The 512x512x257 leg alone (see _leg_512)."""
    import numpy as np
    import torch
    import wvgpu
    from wvgpu import build
    build.build()
    print(json.dumps(_leg_512(wvgpu, torch.cuda.current_stream(), torch, np, args.steps_512)), flush=True)


def run_profile_case(args):
    """A few nonlinear fluxes of the benchmark state, nothing else: the launch
    sequence is vinv, yinv, x products, yfwd, vfwd per flux."""
    import numpy as np
    import torch
    import wvgpu
    from wvgpu import build
    build.build()
    N = args.profile_size
    cfg = configuration(wvgpu) if N == 256 else wvgpu.Configuration(
        Nx=N, Ny=N, Nz=N // 2 + 1, Nj=N // 3, Lx=3125.0 * N, Ly=3125.0 * N, Lz=4000.0, N0=5.2e-3, latitude=33.0)
    k = wvgpu.WVTransformConstantStratificationKernel(cfg, precision=args.profile_flux)
    state = wvgpu.synthetic_state(k, seed=SEED, urms=URMS)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in state]
    out = tuple(torch.empty_like(dev[0]) for _ in range(3))
    torch.cuda.synchronize()
    if args.profile_adjoint:
        dt = wvgpu.cfl_time_step(k, *state)
        k.rk4_adjoint(*dev, 0.0, 0.0, dt, 20, 10, *dev)
        torch.cuda.synchronize()
        print(json.dumps({"profile_adjoint": args.profile_flux, "launches": k.metrics()["kernel_launches"]}))
        k.close()
        return
    for _ in range(args.profile_count):
        k.nonlinearFlux(0.0, 0.0, *dev, out=out)
    if args.profile_vjp:
        for _ in range(args.profile_count):
            k.flux_vjp(0.0, 0.0, *dev, *out)
    torch.cuda.synchronize()
    print(json.dumps({"profile_flux": args.profile_flux, "fluxes": args.profile_count,
                      "launches": k.metrics()["kernel_launches"]}))
    k.close()


def main():
    args = parse()
    if args.profile_flux:
        run_profile_case(args)
    elif args.workload == "512":
        run_workload_512(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
