#!/usr/bin/env python
"""Benchmark of the SEM operator-apply / PCG hot path on one GB300.

Headline (`value`): GDOF/s of the Helmholtz operator with direct-stiffness
summation and Dirichlet mask, mask(QQ'(nu lapl u + lambda B u)), in native FP64
arithmetic, on the 256x256-element, N=8 deformed mesh (4,198,401 unique DOF),
inputs resident in HBM, L2 flushed between steps.  `e2e` is the same metric
through the public API on pinned host buffers (input in, result out every
step).  `df64` is the same apply in the double-float arithmetic (the library's
default operator precision, labelled as such), with its own roofline and e2e.
Extra keys: PCG solves/s (FP64 vs mixed precision), the order sweep
N=4/8/12/16, batched and adjoint solves, the time loop, CPU baselines.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs independent replicas (the path does not shard), one per GPU,
launched by torch.distributed.run; `value` sums all ranks' DOF over the
slowest rank's time.
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
sys.path.insert(0, os.path.join(ROOT, "spectralelements.jl_gb300"))

METRIC = "GDOF/s lapl+QQᵀ; PCG solves/s mixed vs FP64 plain at 1e-8 rel resid, 1 GB300"
UNIT = "GDOF/s"
N_ORDER, E_X, E_Y, AMP, NU, LAM = 8, 256, 256, 0.05, 1e-2, 1.0
BYTES_PER_LOCAL = 48  # u, G11, G12, G22, B read + result written (FP64)
WORKLOAD = ("hlmz+QQ'+mask apply mask(QQ'(nu lapl(u) + lambda B u)), 256x256 elements, N=8 "
            "(9x9 GLL), nu=1e-2, lambda=1, sinusoidal deformation amp 0.05, Dirichlet on all sides")


def sin_deform(amp):
    import numpy as np

    def deform(x, y):
        r = 0.5 * (x + 1.0)
        s = 0.5 * (y + 1.0)
        b = amp * np.sin(np.pi * r) * np.sin(np.pi * s)
        return r + b, s + b
    return deform


def replica_throughput(ms_local, units_per_rank, world, device):
    """Replicas: every rank processes units_per_rank units per step.  Returns
    (step ms = max over ranks, whole-job units per second)."""
    ms = float(ms_local)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * units_per_rank / (ms * 1e-3)


def unique_dof(n, Ex, Ey):
    return (Ex * (n - 1) + 1) * (Ey * (n - 1) + 1)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(name):
    """dram bytes per launch recorded from an ncu capture in profiles/<name>."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid):
        self.uuid = uuid
        self.samples = []
        self.proc = None
        self.marks = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.uuid, f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append((time.time(), parts))

    def mark(self, tag):
        self.marks.append((tag, time.time()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        inside = [p for t, p in self.samples if t0 - 0.25 <= t <= t1 + 0.25]
        use = inside if inside else [p for _, p in self.samples]
        if not use:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(p[0]) for p in use if num(p[0]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for p in use:
            for name, v in zip(names, p[3:7]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": num(use[0][1]),
                "reasons": sorted(reasons), "samples": len(use),
                "window": "timed region" if inside else "whole run (timed region shorter than the 200 ms sampling period)"}


# ---------------------------------------------------------------------------
FP64_OPS_PEAK = 0.625e12  # FP64 pipe instructions/s: DFMA probe, 1.25 TFLOP/s on this machine's GB300
DFMA_PROBE = "DFMA chains, 8 per thread, 1216 CTAs of 256 threads: 1.25 TFLOP/s (0.625 T instr/s)"


def eo_ops(n):
    """FP64 (or double-float) operations of one n-point even-odd line apply."""
    m = n // 2
    return 2 * m + 2 * m * m + (2 * m if n % 2 else 0) + 2 * m


def fp64_ops_per_point(n):
    """Operations per local point of the fused hlmz+QQ'+mask apply in native
    FP64: four line contractions and the metric products (4), or + os (1) and
    the mass term (1; nu is folded into the transposed derivative and k into
    B); the QQ' sums of interface copies are excluded."""
    return 4 * eo_ops(n) / n + 6


def measure_apply(S, lib, msh, prec, u, flush, stream, args, world, dev, G, L, x_pin, y_pin):
    """Time mask(QQ'(hlmz(u))) in one arithmetic: K flushed steps through
    sem_hlmz (device buffers), the operator kernel alone (library CUDA events
    on the launching stream, a second pass), and the end-to-end call on pinned
    host buffers in both modes of sem_hlmz_host."""
    import ctypes

    import torch
    msh.set_precision(prec)
    sp = stream.cuda_stream
    flags = S.SEM_GS | S.SEM_MASK
    out = msh.empty()

    def apply():
        S._lib.check(lib.sem_hlmz(msh.handle, None, NU, LAM, u.data_ptr(), out.data_ptr(), flags, sp))

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        flush.fill_(1.0)
        apply()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    t0 = time.time()
    torch.cuda.nvtx.range_push("timed")  # the launch-list filter of a profiler run
    for i in range(args.steps):
        flush.fill_(float(i))  # L2 flush (512 MiB write), outside the timed events
        ev[i][0].record(stream)
        apply()
        ev[i][1].record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    t1 = time.time()
    lib.sem_timing_read(None, None)
    lib.sem_timing_enable(1)
    for i in range(args.steps):
        flush.fill_(float(i))
        apply()
    torch.cuda.synchronize()
    lib.sem_timing_enable(0)
    kms, kn = ctypes.c_double(), ctypes.c_int()
    lib.sem_timing_read(ctypes.byref(kms), ctypes.byref(kn))
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms, per_s = replica_throughput(sum(step_ms) / len(step_ms), G, world, dev)
    kernel_ms = kms.value / max(1, kn.value)
    # end to end: pinned host buffers in and out every step, in the two modes
    # of the host-buffer call (copy-engine slabs; kernels reading and writing
    # the host buffers in place); the faster is reported
    op = S.HelmholtzOp(msh, NU, LAM)
    modes = {}
    for mode_name, slabs in (("8 copy-engine slabs overlapped with the kernels", 8),
                             ("kernels read and write the host buffers in place", S._lib.SEM_HOST_DIRECT)):
        e2e_ms = []
        for i in range(args.warmup + args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            op.apply_host(x_pin, y_pin, slabs=slabs)
            b.record(stream)
            b.synchronize()
            if i >= args.warmup:
                e2e_ms.append(a.elapsed_time(b))
        modes[mode_name] = (sum(e2e_ms) / len(e2e_ms), slabs)
    best = min(modes, key=lambda k: modes[k][0])
    e2e_step, e2e_per_s = replica_throughput(modes[best][0], G, world, dev)
    op.apply_host(x_pin, y_pin, slabs=modes[best][1])
    torch.cuda.synchronize()
    y_dev = op(u)
    e2e = {"value": e2e_per_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": 8 * L, "d2h_bytes_per_step": 8 * L,
           "ms_per_step": e2e_step,
           "api": "semgb300.HelmholtzOp.apply_host (sem_hlmz_host through ctypes), pinned host buffers: " + best,
           "ms_per_mode": {k: v[0] for k, v in modes.items()},
           "matches_device_call": bool(torch.equal(y_pin, y_dev.cpu()))}
    return {"value": per_s / 1e9, "ms": ms, "kernel_ms": kernel_ms, "kernel_launches": kn.value,
            "e2e": e2e, "t0": t0, "t1": t1, "y": y_dev}


def kernel_name(prec_tag, variant):
    kname = ("k_apply", "k_apply", "k_apply2", "k_apply2", "k_apply3", "k_apply2", "k_apply4")[variant]
    targs = {0: "false", 1: "true", 2: "false,false,false", 3: "true,false,false", 4: None,
             5: "false,true,false", 6: None}[variant]
    return f"{kname}<{prec_tag},9,8,3{',' + targs if targs else ''}>"


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    import semgb300 as S

    torch.cuda.set_device(local_rank)
    lib = S.load()
    dev = torch.device("cuda", local_rank)
    uuid = str(torch.cuda.get_device_properties(dev).uuid)
    sampler = ClockSampler(uuid if uuid.startswith("GPU-") else "GPU-" + uuid)
    sampler.start()

    msh = S.Mesh(N_ORDER + 1, N_ORDER + 1, E_X, E_Y, (False, False), sin_deform(AMP), bc="DDDD")
    tune = {name: msh.autotune(prec) for name, prec in
            (("f64", S.SEM_F64), ("df64", S.SEM_F64_DF), ("f32", S.SEM_F32))}
    if args.variant is not None:
        # a pinned FP64 kernel variant (profiling runs, where the autotuner's
        # timings are distorted by the profiler)
        msh.set_variant(args.variant, S.SEM_F64)
        tune["f64"]["chosen"] = args.variant
        tune["f64"]["pinned"] = True
    nx, ny = msh.shape
    L = nx * ny
    G = unique_dof(N_ORDER + 1, E_X, E_Y)
    rng = np.random.default_rng(3)
    u_h = rng.uniform(-1.0, 1.0, (nx, ny))
    u = S.as_local(u_h)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    x_pin = torch.empty_strided((nx, ny), (1, nx), dtype=torch.float64, pin_memory=True)
    x_pin.copy_(torch.from_numpy(np.asfortranarray(u_h)))
    y_pin = torch.empty_strided((nx, ny), (1, nx), dtype=torch.float64, pin_memory=True)

    head = measure_apply(S, lib, msh, S.SEM_F64, u, flush, stream, args, world, dev, G, L, x_pin, y_pin)
    clocks = sampler.summary(head["t0"], head["t1"])
    df64 = None
    if world == 1:
        df64 = measure_apply(S, lib, msh, S.SEM_F64_DF, u, flush, stream, args, world, dev, G, L, x_pin, y_pin)
    peak, peak_kind = load_peaks()
    bytes_launch = BYTES_PER_LOCAL * L
    ops_launch = fp64_ops_per_point(N_ORDER + 1) * L

    def roof(m, tag, variant, prof):
        achieved = bytes_launch / (m["kernel_ms"] * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": profiled_traffic(prof),
                "kernel": kernel_name(tag, variant) + f" (fused element operator, autotuned variant {variant})",
                "kernel_ms": m["kernel_ms"], "kernel_launches_timed": m["kernel_launches"],
                "kernel_timing": "CUDA events around each operator launch on its stream, in a second pass of the "
                                 "same K flushed steps right after the timed region",
                "algorithmic_bytes_per_launch": bytes_launch}

    v64 = tune["f64"]["chosen"]
    roofline = roof(head, "PF64", v64, "k_apply_hlmz_f64_256x256_n8.md")
    ops_s = ops_launch / (head["kernel_ms"] * 1e-3)
    roofline["fp64_pipe"] = {"achieved_instr_per_s": ops_s, "peak_instr_per_s": FP64_OPS_PEAK,
                             "frac": ops_s / FP64_OPS_PEAK, "peak_source": DFMA_PROBE,
                             "fp64_instr_per_launch": ops_launch,
                             "note": "the kernel's bound on GB300: FP64 runs at 1/64 of the FP32 rate, so "
                                     "native FP64 caps this apply far below the HBM roofline"}
    result = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded U(-1,1) field (seed 3) on the seeded deformed mesh",
        "config": {"workload": WORKLOAD, "elements": [E_X, E_Y], "order": N_ORDER,
                   "unique_dof": G, "local_dof": L,
                   "arith": "native FP64 (SEM_F64): every operation an IEEE double instruction",
                   "l2": "flushed between timed steps (512 MiB write outside the events)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "autotune": tune},
        "roofline": roofline, "e2e": head["e2e"],
        "gpu_launches": (1 if v64 == 5 else 2) * args.steps, "clocks": clocks,
    }
    if df64 is not None:
        vdf = tune["df64"]["chosen"]
        rel = (torch.linalg.norm(df64["y"] - head["y"]) / torch.linalg.norm(head["y"])).item()
        result["df64"] = {
            "arith": "double-float: each value an unevaluated sum of two FP32 numbers (about 47 significand "
                     "bits, FP32 exponent range; element tiles whose inputs or intermediates leave the pair "
                     "format's range are recomputed in native FP64 inside the kernel); FP64 storage",
            "value": df64["value"], "unit": UNIT, "ms_per_step": df64["ms"], "rel_l2_vs_f64": rel,
            "roofline": roof(df64, "PDF", vdf, f"{kernel_name('PDF', vdf).split('<')[0]}_hlmz_df_256x256_n8.md"),
            "e2e": df64["e2e"]}
        result["f32_inner_operator"] = {"ms": tune["f32"]["ms"][tune["f32"]["chosen"]],
                                        "note": "FP32 operator of the mixed-precision inner CG (autotune time)"}
    if not args.no_extras and world == 1:  # the N-replica runs measure the headline only
        extras = args.extras.split(",") if args.extras else ["pcg", "sweep", "batch", "adjoint", "time"]
        msh.set_precision(S.SEM_F64_DF)
        if "pcg" in extras:
            result["pcg"] = bench_pcg(S, msh, stream)
        elif "small" in extras:  # cfg1/cfg3 only
            result["pcg"] = bench_pcg(S, msh, stream, parts=("small",))
        if "sweep" in extras:
            result["sweep"] = bench_sweep(S, stream)
        if "batch" in extras:
            result["batch"] = bench_batch(S)
        if "adjoint" in extras:
            result["adjoint"] = bench_adjoint(S, args.fd_directions)
        if "time" in extras:
            result["time"] = bench_time(S)
    sampler.stop()
    if rank == 0 and world == 1 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(result.get("pcg"), result.get("batch"), result.get("adjoint"))
    if "batch" in result:
        result["batch"].pop("_problems", None)
    return result


def time_apply(fn, stream, reps):
    import torch
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / reps


def fourier_forcing(msh_x, msh_y, seed, nmodes=16):
    import numpy as np
    import torch
    rng = np.random.default_rng(seed)
    f = torch.zeros_like(msh_x)
    for _ in range(nmodes):
        kx, ky = rng.integers(1, 9, size=2)
        c = rng.standard_normal() / (kx ** 2 + ky ** 2)
        f += c * torch.sin(float(kx) * np.pi * msh_x) * torch.sin(float(ky) * np.pi * msh_y)
    return f


def bench_pcg(S, msh, stream, parts=("cfg2", "small")):
    """Jacobi PCG to 1e-8 relative residual: native FP64, double-float (FP64
    storage, FP32-pair arithmetic) and mixed precision (FP32 inner CG to
    1e-4, <= 6 FP64 defect-correction sweeps; or residual replacement).
    ``parts``: "cfg2" (256x256) and "small" (cfg1/cfg3, 8x8)."""
    import numpy as np
    import torch
    out = {}
    if "cfg2" in parts:
        bench_pcg_cfg2(S, msh, out)
    if "small" in parts:
        bench_pcg_small(S, out)
    return out


def bench_pcg_cfg2(S, msh, out):
    import numpy as np
    import torch
    # cfg2: Helmholtz 256x256, N=8, 16 Fourier modes (seed 2)
    f = fourier_forcing(msh.x, msh.y, 2)
    M = S.generateMask("DDDD", msh)
    b = S.gatherScatter(S.mask(S.mass(f, msh), M), msh)
    tol = 1e-8 * b.abs().max().item()
    op = S.HelmholtzOp(msh, NU, LAM)
    jac = S.Jacobi(op)
    res = {}
    msh.autotune(S.SEM_F64)
    for name, prec in (("fp64", S.SEM_F64), ("df64", S.SEM_F64_DF), ("mixed", S.SEM_MIXED),
                       ("mixed_rr", S.SEM_MIXED_RR)):
        info = {}
        S.pcg(b, op, opM=jac, mult=msh.mult, tol=tol, precision=prec, info=info)  # warm
        torch.cuda.synchronize()
        t = time.time()
        x = S.pcg(b, op, opM=jac, mult=msh.mult, tol=tol, precision=prec, info=info)
        torch.cuda.synchronize()
        dt = time.time() - t
        res[name] = (x, dt, dict(info))
    x64, dt64, i64 = res["fp64"]

    def rel(x):
        return (torch.linalg.norm(x - x64) / torch.linalg.norm(x64)).item()

    xd, dtd, idf = res["df64"]
    xm, dtm, im = res["mixed"]
    xr, dtr, ir = res["mixed_rr"]
    out["cfg2_helmholtz_256x256_n8"] = {
        "tol_rel": 1e-8,
        "fp64": {"solves_per_s": 1 / dt64, "iters": i64["iters"], "res_inf": i64["res_inf"],
                 "res0_inf": i64["res0_inf"], "arith": "native FP64 operator, vectors and dots"},
        "df64": {"solves_per_s": 1 / dtd, "iters": idf["iters"], "res_inf": idf["res_inf"],
                 "rel_l2_vs_fp64": rel(xd),
                 "arith": "double-float operator (FP32 pairs, about 47 bits), FP64 vectors, double-float dots"},
        "mixed": {"solves_per_s": 1 / dtm, "inner_iters": im["iters"], "outer": im["outer"],
                  "res_inf": im["res_inf"], "rel_l2_vs_fp64": rel(xm),
                  "form": "FP32 inner CG to 1e-4 relative, restarted, inside FP64 defect-correction sweeps"},
        "mixed_rr": {"solves_per_s": 1 / dtr, "iters": ir["iters"], "replacements": ir["outer"],
                     "res_inf": ir["res_inf"], "rel_l2_vs_fp64": rel(xr),
                     "form": "one FP32 CG; its residual replaced by the FP64 b - A x (x in FP64) "
                             "whenever it has fallen by 0.3; search direction kept"},
        "mixed_over_fp64": dt64 / dtm, "mixed_rr_over_fp64": dt64 / dtr,
        "mixed_over_df64": dtd / dtm, "mixed_rr_over_df64": dtd / dtr}


def bench_pcg_small(S, out):
    import numpy as np
    import torch
    # cfg1 / cfg3: Poisson 8x8, N=8, amp 0.1, exact solution sin(pi x) sin(pi y), 1e-10
    m1 = S.Mesh(9, 9, 8, 8, (False, False), sin_deform(0.1), bc="DDDD")
    m1.autotune(S.SEM_F64_DF)
    m1.autotune(S.SEM_F32)
    ut = torch.sin(np.pi * m1.x) * torch.sin(np.pi * m1.y)
    f1 = 2 * np.pi ** 2 * ut
    M1 = S.generateMask("DDDD", m1)
    b1 = S.gatherScatter(S.mask(S.mass(f1, m1), M1), m1)
    op1 = S.HelmholtzOp(m1, 1.0, 0.0)
    jac1 = S.Jacobi(op1)
    r = {}
    m1.autotune(S.SEM_F64)
    for name, prec, tolr in (("cfg1_fp64", S.SEM_F64, 1e-10), ("cfg1_df64", S.SEM_F64_DF, 1e-10),
                             ("cfg3_mixed", S.SEM_MIXED, 1e-10),
                             ("cfg3_mixed_1e-8", S.SEM_MIXED, 1e-8), ("cfg1_fp64_1e-8", S.SEM_F64, 1e-8),
                             ("cfg3_mixed_rr", S.SEM_MIXED_RR, 1e-10), ("cfg3_mixed_rr_1e-8", S.SEM_MIXED_RR, 1e-8)):
        tol1 = tolr * b1.abs().max().item()
        info = {}
        S.pcg(b1, op1, opM=jac1, mult=m1.mult, tol=tol1, precision=prec, info=info)
        torch.cuda.synchronize()
        reps = 20
        t = time.time()
        for _ in range(reps):
            x = S.pcg(b1, op1, opM=jac1, mult=m1.mult, tol=tol1, precision=prec, info=info)
        torch.cuda.synchronize()
        dt = (time.time() - t) / reps
        r[name] = {"solves_per_s": 1 / dt, "iters": info["iters"], "outer": info["outer"],
                   "res_inf": info["res_inf"], "tol_rel": tolr,
                   "err_vs_exact_inf": (x - ut).abs().max().item()}
    r["cfg3_mixed_over_cfg1_fp64"] = r["cfg3_mixed"]["solves_per_s"] / r["cfg1_fp64"]["solves_per_s"]
    r["cfg3_mixed_over_cfg1_df64"] = r["cfg3_mixed"]["solves_per_s"] / r["cfg1_df64"]["solves_per_s"]
    r["note"] = ("cfg1_fp64: native FP64 arithmetic throughout; cfg1_df64: double-float operator and dots; "
                 "cfg3_mixed: FP32 inner CG in one thread block, double-float FP64 residual sweeps")
    out["cfg1_cfg3_poisson_8x8_n8"] = r


def d2d_problem(S, msh):
    """examples/d2d.jl:13-33 on msh: u = sin(2 pi x) sin(2 pi y) cos(2 pi t) with
    its forcing split into two separable modes (spatial field, coefficient of t)."""
    import numpy as np
    import torch
    k = 2.0
    sp = torch.sin(k * np.pi * msh.x) * torch.sin(k * np.pi * msh.y)
    modes = [(sp * (2 * k * k * np.pi ** 2), lambda t: float(np.cos(k * np.pi * t))),
             (sp * (-k * np.pi), lambda t: float(np.sin(k * np.pi * t)))]
    return sp, modes


def bench_time(S):
    """The Diffusion driver (src/diffusion.jl:81-137): BDF3, dt = 1e-3, the
    reference's solve (identity preconditioner, mult-weighted dots, absolute
    tol 1e-8), d2d.jl's manufactured solution.  One sem_bdf_run call for the
    whole run against the per-step evolve() loop with a setForcing! closure,
    as the reference's examples drive it."""
    import numpy as np
    import torch
    out = {}
    for name, E, steps, loop_steps in (("cfg1_mesh_8x8_n8", 8, 1000, 200), ("mesh_64x64_n8", 64, 100, 40)):
        m = S.Mesh(9, 9, E, E, (False, False), sin_deform(0.1), bc="DDDD")
        m.autotune(S.SEM_F64_DF)
        sp, modes = d2d_problem(S, m)
        r = {"steps": steps, "dt": 1e-3, "order": 3, "tol_abs": 1e-8,
             "local_dof": int(m.x.numel()), "path": "small (one cluster launch per solve)"
             if m.x.numel() <= S._lib.SEM_SMALL_MAX_LOCAL else "chunked (CUDA-graph CG chunks)"}
        # device-resident run
        d = S.Diffusion("DDDD", m, Ti=0.0, Tf=1.0, dt=1e-3, k=3, nu=1.0)
        d.u.copy_(sp)
        d.run(5, forcing=modes)  # warm
        d = S.Diffusion("DDDD", m, Ti=0.0, Tf=1.0, dt=1e-3, k=3, nu=1.0)
        d.u.copy_(sp)
        torch.cuda.synchronize()
        t = time.time()
        infos = d.run(steps, forcing=modes)
        torch.cuda.synchronize()
        dt_run = time.time() - t
        err = (d.u - sp * np.cos(2 * np.pi * d.tstep.time[0])).abs().max().item()
        r["device_run"] = {"steps_per_s": steps / dt_run, "iters_per_step": sum(i["iters"] for i in infos) / steps,
                           "err_vs_exact_inf": err}
        # per-step evolve loop (host closure sets f each step)
        e = S.Diffusion("DDDD", m, Ti=0.0, Tf=1.0, dt=1e-3, k=3, nu=1.0)
        e.u.copy_(sp)
        a0, a1 = modes[0][0], modes[1][0]

        def set_f(f, x, y, tt):
            f.copy_(modes[0][1](tt) * a0 + modes[1][1](tt) * a1)
        e.evolve(setForcing=set_f)
        torch.cuda.synchronize()
        t = time.time()
        for _ in range(loop_steps):
            e.evolve(setForcing=set_f)
        torch.cuda.synchronize()
        dt_loop = time.time() - t
        r["evolve_loop"] = {"steps_per_s": loop_steps / dt_loop, "steps": loop_steps}
        r["run_over_loop"] = (steps / dt_run) / (loop_steps / dt_loop)
        out[name] = r
    return out


def bench_batch(S):
    """cfg4: 512 independent Helmholtz problems (seed 4): Ex, Ey ~ U{4..64},
    N ~ U{4,6,8,10}, nu log-uniform in [1e-3, 1], lambda ~ U[0, 10], deformation
    amplitude 0.05, forcing 2 pi^2 sin(pi x) sin(pi y), Dirichlet, Jacobi, tol
    1e-8 relative; one persistent launch per order.  Also cfg1/cfg3 (one
    8x8 N=8 Poisson problem) through the same persistent kernel."""
    import numpy as np
    import torch
    rng = np.random.default_rng(4)
    meshes, nus, lams, bs, tols, shapes = [], [], [], [], [], []
    for _ in range(512):
        Ex, Ey = (int(v) for v in rng.integers(4, 65, size=2))
        N = int(rng.choice([4, 6, 8, 10]))
        nus.append(float(10 ** rng.uniform(-3, 0)))
        lams.append(float(rng.uniform(0, 10)))
        shapes.append((N, Ex, Ey))
        m = S.Mesh(N + 1, N + 1, Ex, Ey, (False, False), sin_deform(0.05), bc="DDDD")
        f = 2 * np.pi ** 2 * torch.sin(np.pi * m.x) * torch.sin(np.pi * m.y)
        M = S.generateMask("DDDD", m)
        b = S.gatherScatter(S.mask(S.mass(f, m), M), m)
        meshes.append(m)
        bs.append(b)
        tols.append(1e-8 * b.abs().max().item())
    local = sum(m.shape[0] * m.shape[1] for m in meshes)
    solver = S.BatchSolver(meshes, nus, lams, jacobi=True)
    out = {"problems": 512, "local_dof": local,
           "arith": {"df64": "double-float operator and dots (FP32 pairs, about 47 bits), FP64 vectors; "
                             "the batch kernels have no native-FP64 form",
                     "mixed": "FP32 inner CG inside FP64 defect-correction sweeps",
                     "mixed_rr": "FP32 CG with FP64 residual replacement"}}
    default_cfg, default_order = solver.config(), solver.order()
    # the autotuner's choices persist per batch signature (device, arithmetic,
    # every problem's shape, coefficients and tolerance) in the package's
    # cache file; a signature found there is loaded without solving
    cache = os.path.join(ROOT, "spectralelements.jl_gb300", "semgb300", "tuned", "batch.txt")
    os.makedirs(os.path.dirname(cache), exist_ok=True)

    def timed(prec):
        infos = []
        torch.cuda.synchronize()
        t = time.time()
        x = solver.solve(bs, tols, precision=prec, infos=infos)
        torch.cuda.synchronize()
        return x, time.time() - t, infos

    def timeline_summary():
        tl = solver.timeline()
        busy = {}
        for s0, s1, c in zip(tl["start_ns"], tl["end_ns"], tl["cluster"]):
            if c >= 0:
                busy.setdefault(int(c), []).append((int(s0), int(s1)))
        ends = sorted(max(e for _, e in v) for v in busy.values())
        per = sorted(sum(e - b for b, e in v) for v in busy.values())
        span = max(ends) if ends else 0
        return {"device_ms": tl["total_ms"], "clusters_seen": len(busy), "makespan_ms": span / 1e6,
                "cluster_busy_ms": {"min": per[0] / 1e6, "median": per[len(per) // 2] / 1e6, "max": per[-1] / 1e6},
                "first_cluster_done_ms": ends[0] / 1e6,
                "busy_fraction": sum(per) / (span * len(per)) if span else 0.0}

    xs = {}
    for name, prec in (("df64", S.SEM_F64_DF), ("mixed", S.SEM_MIXED), ("mixed_rr", S.SEM_MIXED_RR)):
        solver.set_config(default_cfg)
        solver.set_order(default_order)
        solver.set_wide([0] * len(meshes))
        solver.solve(bs, tols, precision=prec)  # warm
        x0, dt0, infos = timed(prec)
        tl0 = timeline_summary()
        t = time.time()
        tune = solver.autotune(bs, tols, precision=prec, cache=cache)
        tune_s = time.time() - t
        xs[name], dt, infos = timed(prec)
        it = [i["iters"] for i in infos]
        out[name] = {"batch_s": dt, "solves_per_s": 512 / dt, "converged": sum(i["converged"] for i in infos),
                     "iters_max": max(it), "iters_mean": float(np.mean(it)),
                     "tuned_config": [{k: c[k] for k in ("n", "problems", "cluster_size", "ctas_per_sm", "clusters")}
                                      for c in tune["config"]],
                     "wide_problems": sum(tune["wide"]),
                     "tune": {"solves": tune["runs"], "seconds": tune_s,
                              "source": "loaded from the tuning cache" if tune["runs"] == 0 else "tuned now"},
                     "timeline": timeline_summary(),
                     "default": {"batch_s": dt0, "solves_per_s": 512 / dt0,
                                 "config": "cluster_size 8, ctas_per_sm 2, work-proportional cluster counts, "
                                           "estimated-work order", "timeline": tl0}}
        if name == "df64":  # per-problem record for the CPU baseline's sample (not printed)
            out["_problems"] = [{"N": N, "Ex": Ex, "Ey": Ey, "nu": nu, "lam": lam, "iters": i,
                                 "local": (N + 1) ** 2 * Ex * Ey}
                                for (N, Ex, Ey), nu, lam, i in zip(shapes, nus, lams, it)]
    for name in ("mixed", "mixed_rr"):
        errs = [(torch.linalg.norm(a - b) / torch.linalg.norm(b)).item() for a, b in zip(xs[name], xs["df64"])]
        out[name]["rel_l2_vs_df64_max"] = max(errs)
        out[name + "_over_df64"] = out["df64"]["batch_s"] / out[name]["batch_s"]
    del solver, meshes, bs, xs
    # cfg1 / cfg3 through the persistent kernel (one cluster, one problem)
    m1 = S.Mesh(9, 9, 8, 8, (False, False), sin_deform(0.1), bc="DDDD")
    ut = torch.sin(np.pi * m1.x) * torch.sin(np.pi * m1.y)
    M1 = S.generateMask("DDDD", m1)
    b1 = S.gatherScatter(S.mask(S.mass(2 * np.pi ** 2 * ut, m1), M1), m1)
    one = S.BatchSolver([m1], [1.0], [0.0], jacobi=True)
    res = {}
    for name, prec, tolr in (("cfg1_df64", S.SEM_F64_DF, 1e-10), ("cfg3_mixed", S.SEM_MIXED, 1e-10)):
        tol1 = [tolr * b1.abs().max().item()]
        infos = []
        one.solve([b1], tol1, precision=prec, infos=infos)
        torch.cuda.synchronize()
        reps = 50
        t = time.time()
        for _ in range(reps):
            x = one.solve([b1], tol1, precision=prec, infos=infos)[0]
        torch.cuda.synchronize()
        dt = (time.time() - t) / reps
        res[name] = {"solves_per_s": 1 / dt, "iters": infos[0]["iters"], "outer": infos[0]["outer"],
                     "err_vs_exact_inf": (x - ut).abs().max().item()}
    out["cfg1_cfg3_persistent"] = res
    return out


def gaussian_field(x, y, seed, sigma=0.5, nk=8):
    """Seeded smooth random field: sum over kx, ky <= nk of N(0,1) k^-2
    cos/sin modes with random phases, normalised to standard deviation sigma."""
    import numpy as np
    rng = np.random.default_rng(seed)
    g = np.zeros(x.shape)
    for kx in range(1, nk + 1):
        for ky in range(1, nk + 1):
            a, b = rng.standard_normal(2) / (kx * kx + ky * ky)
            ph = rng.uniform(0, 2 * np.pi)
            g += a * np.cos(np.pi * (kx * x + ky * y) + ph) + b * np.sin(np.pi * (kx * x - ky * y))
    return sigma * (g - g.mean()) / g.std()


def bench_adjoint(S, fd_directions):
    """cfg5: steady -div(nu grad u) = 1 on 128x128 elements, N=8, Dirichlet,
    nu = exp(g) (seed 5), J = 1/2 sum B (u - u_target)^2 (u_target seed 6);
    gradient w.r.t. the nodal nu by the adjoint solve (autograd function over
    sem_pcg + sem_adjoint_grad), checked by central differences (h = 1e-6,
    continuous random directions, seed 7; native FP64 J evaluations); then 200
    implicit-Euler steps (dt = 1e-3) forward and backward with checkpoints
    every 20 steps."""
    import numpy as np
    import torch
    msh = S.Mesh(9, 9, 128, 128, (False, False), sin_deform(0.05), bc="DDDD")
    x = msh.x.cpu().numpy()
    y = msh.y.cpu().numpy()
    nu = torch.from_numpy(np.exp(gaussian_field(x, y, 5))).cuda()
    nu = S.as_local(nu)
    ut = S.as_local(torch.from_numpy(0.05 * gaussian_field(x, y, 6)).cuda())
    M = S.generateMask("DDDD", msh)
    b = S.gatherScatter(S.mask(S.mass(torch.ones_like(msh.x), msh), M), msh)
    tol = 1e-12 * b.abs().max().item()
    B = msh.B
    out = {"mesh": "128x128 elements, N=8", "tol_rel": 1e-12}

    def gradient(**kw):
        nu_t = nu.clone().requires_grad_(True)
        u = S.linsolve_varcoef(nu_t, b, msh, tol=tol, **kw)
        J = 0.5 * torch.sum(B * (u - ut) ** 2)
        J.backward()
        return J.item(), nu_t.grad

    gradient()  # warm
    torch.cuda.synchronize()
    t = time.time()
    J0, g = gradient()
    torch.cuda.synchronize()
    out["gradient_s"] = time.time() - t
    out["J"] = J0
    # iteration counts of the forward and the adjoint solve (for the CPU baseline)
    opv = S.HelmholtzOp(msh, 1.0, 0.0, nu_field=nu)
    i_f, i_a = {}, {}
    u0v = S.pcg(b, opv, opM=S.Jacobi(opv), mult=msh.mult, tol=tol, info=i_f)
    rhs_a = S.gatherScatter(S.mask(B * (u0v - ut), M), msh)
    S.pcg(rhs_a, opv, opM=S.Jacobi(opv), mult=msh.mult, tol=tol, info=i_a)
    out["forward_iters"], out["adjoint_iters"] = i_f["iters"], i_a["iters"]

    # central finite differences along continuous directions
    msh.set_precision(S.SEM_F64)

    def J_of(nu_v):
        u = S.linsolve_varcoef(nu_v, b, msh, tol=tol)
        return 0.5 * torch.sum(B * (u - ut) ** 2).item()

    gen = torch.Generator(device="cuda").manual_seed(7)
    errs = []
    h = 1e-6
    t = time.time()
    for _ in range(fd_directions):
        delta = msh.mult * S.gatherScatter(S.as_local(torch.randn(msh.shape, generator=gen, device="cuda",
                                                                  dtype=torch.float64)), msh)
        fd = (J_of(nu + h * delta) - J_of(nu - h * delta)) / (2 * h)
        ad = torch.sum(g * delta).item()
        errs.append(abs(fd - ad) / abs(ad))
    out["fd"] = {"directions": fd_directions, "h": h, "max_rel_err": max(errs),
                 "median_rel_err": float(np.median(errs)), "s": time.time() - t}
    msh.set_precision(S.SEM_F64_DF)
    # transient: 200 implicit-Euler steps with checkpoints every 20
    u0 = S.mask(torch.sin(np.pi * msh.x) * torch.sin(np.pi * msh.y), M)
    f = torch.ones_like(msh.x)
    dt, steps, every = 1e-3, 200, 20
    nu_t = nu.clone().requires_grad_(True)
    # tolerance relative to the first step's right-hand side B u0 / dt + B f
    rhs0 = S.gatherScatter(S.mask(S.mass(u0, msh), M), msh) / dt + b
    tol_t = 1e-10 * rhs0.abs().max().item()
    torch.cuda.synchronize()
    t = time.time()
    uT = S.transient_varcoef(nu_t, u0, f, msh, dt, steps, every, tol=tol_t)
    torch.cuda.synchronize()
    t_fwd = time.time() - t
    J = 0.5 * torch.sum(B * (uT - ut) ** 2)
    t = time.time()
    J.backward()
    torch.cuda.synchronize()
    t_bwd = time.time() - t
    # CG iterations of the first step's solve (each step is a cold-started CG)
    op1 = S.HelmholtzOp(msh, 1.0, 1.0 / dt, nu_field=nu)
    info1 = {}
    S.pcg(rhs0, op1, opM=S.Jacobi(op1), mult=msh.mult, tol=tol_t, info=info1)
    out["transient"] = {"steps": steps, "dt": dt, "checkpoint_every": every, "forward_s": t_fwd,
                        "backward_s": t_bwd, "first_step_iters": info1["iters"],
                        "grad_finite": bool(torch.isfinite(nu_t.grad).all().item())}
    return out


def bench_sweep(S, stream):
    """Apply GDOF/s across orders at ~4M unique DOF (double-float, L2-resident
    inputs larger than L2)."""
    import numpy as np
    import torch
    res = {}
    for N, E in ((4, 500), (8, 256), (12, 167), (16, 125)):
        m = S.Mesh(N + 1, N + 1, E, E, (False, False), sin_deform(AMP), bc="DDDD")
        tv = m.autotune()
        u = S.as_local(torch.rand(m.shape, dtype=torch.float64, device="cuda") * 2 - 1)
        op = S.HelmholtzOp(m, NU, LAM)
        ms = time_apply(lambda: op(u), stream, 10)
        G = unique_dof(N + 1, E, E)
        L = (N + 1) ** 2 * E * E
        res[f"N{N}_E{E}"] = {"GDOF/s": G / (ms * 1e-3) / 1e9, "ms": ms, "variant": tv["chosen"],
                             "GB/s_alg": BYTES_PER_LOCAL * L / (ms * 1e-3) / 1e9}
        del m
    return res


# ---------------------------------------------------------------------------
def reference_apply_timer(threads_note=True):
    """The reference's CPU path, restated in NumPy (reference-faithful: dense
    QQtx/QQty as the reference's Mesh stores them, BLAS gemms in ABu)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import sem_oracle as O
    mo = O.Mesh(N_ORDER + 1, N_ORDER + 1, E_X, E_Y, (False, False), O.sin_deform(AMP), dense_qq=True)
    M = O.generateMask(["D"] * 4, mo)
    rng = np.random.default_rng(3)
    u = rng.uniform(-1.0, 1.0, mo.shape)

    def step():
        return O.mask(O.gatherScatter(O.hlmz(u, NU, LAM, mo), mo), M)
    return step, mo


def cpu_baseline(pcg=None, batch=None, adjoint=None):
    """Bounded CPU samples on the host cores: the reference-faithful NumPy
    restatement (kind 'port') of the apply and of the solves, plus the
    optimised C/OpenMP oracle."""
    import numpy as np
    step, mo = reference_apply_timer()
    step()
    times = []
    t_end = time.time() + 12.0
    while time.time() < t_end or len(times) < 2:
        t = time.time()
        step()
        times.append(time.time() - t)
        if len(times) >= 10:
            break
    G = unique_dof(N_ORDER + 1, E_X, E_Y)
    val = G / statistics.median(times) / 1e9
    out = {"value": val, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
           "sample": f"{len(times)} applies of the full 256x256 N=8 workload, reference-faithful "
                     "NumPy restatement (dense QQtx/QQty gemms as src/mesh.jl:44-45 stores them, "
                     "BLAS threads = all host cores); median",
           "ms_per_apply": 1e3 * statistics.median(times)}
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import sem_oracle_c as C
        g = C.grid(N_ORDER + 1, E_X, E_Y, (False, False), "DDDD")
        rng = np.random.default_rng(3)
        u = rng.uniform(-1.0, 1.0, mo.shape)
        C.apply(g, mo.Dr, mo.Ds, mo.G11, mo.G12, mo.G22, mo.B, u, nu=NU, k=LAM)
        ts = []
        for _ in range(5):
            t = time.time()
            C.apply(g, mo.Dr, mo.Ds, mo.G11, mo.G12, mo.G22, mo.B, u, nu=NU, k=LAM)
            ts.append(time.time() - t)
        out["optimised_c_openmp"] = {"value": G / statistics.median(ts) / 1e9, "unit": UNIT,
                                     "threads": C.threads(), "ms_per_apply": 1e3 * statistics.median(ts)}
    except Exception as e:  # the C oracle is optional for the baseline line
        out["optimised_c_openmp"] = {"error": str(e)}
    out["time_loop_cfg1_mesh_8x8_n8"] = cpu_time_loop()
    try:
        out["solves"] = cpu_solve_baselines(pcg, batch, adjoint)
    except Exception as e:
        out["solves"] = {"error": str(e)}
    return out


def cpu_solve_baselines(pcg=None, batch=None, adjoint=None):
    """Solves/s of the reference's CPU path (src/pcg.jl:16-60 on
    src/diffusion.jl:36-45's operator) for each configuration, on bounded
    samples: the reference-faithful NumPy restatement (dense QQ', the port)
    and the C/OpenMP oracle (sum-factorised).  Where a full solve would take
    minutes, the time of a few iterations is multiplied by the iteration
    count of the GPU solve of the same problem, and the entry says so."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import sem_oracle as O
    import sem_oracle_c as C
    res = {"cores": os.cpu_count(), "threads_c": C.threads()}

    def port_solver(mo, nu, k, M, d):
        return lambda b, tol, maxiter=None, info=None: O.pcg(
            b, lambda v: O.mask(O.gatherScatter(O.hlmz(v, nu, k, mo), mo), M),
            opM=lambda r: r / d, mult=mo.mult, tol=tol, maxiter=maxiter, info=info)

    # cfg1: Poisson 8x8, N=8, amp 0.1, Jacobi PCG to 1e-10 relative (full solves)
    mo = O.Mesh(9, 9, 8, 8, (False, False), O.sin_deform(0.1), dense_qq=True)
    M = O.generateMask(["D"] * 4, mo)
    f = 2 * np.pi ** 2 * np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y)
    b = O.gatherScatter(O.mask(O.mass(f, mo), M), mo)
    tol = 1e-10 * np.abs(b).max()
    d = O.jacobi_diag(mo, 1.0, 0.0, M)
    solve = port_solver(mo, 1.0, 0.0, M, d)
    info = {}
    solve(b, tol, info=info)
    n, t0 = 0, time.time()
    while time.time() - t0 < 3.0 or n < 2:
        solve(b, tol)
        n += 1
    port1 = n / (time.time() - t0)
    g1 = C.grid(9, 8, 8, (False, False), "DDDD")
    C.pcg(g1, mo.Dr, mo.Ds, mo.G11, mo.G12, mo.G22, mo.B, b, nu=1.0, k=0.0, d=d, tol=tol)
    n, t0 = 0, time.time()
    while time.time() - t0 < 2.0 or n < 2:
        _, it1, _ = C.pcg(g1, mo.Dr, mo.Ds, mo.G11, mo.G12, mo.G22, mo.B, b, nu=1.0, k=0.0, d=d, tol=tol)
        n += 1
    c1 = n / (time.time() - t0)
    res["cfg1_poisson_8x8_n8_1e-10"] = {"port_solves_per_s": port1, "port_iters": info.get("iters"),
                                        "c_openmp_solves_per_s": c1, "c_iters": it1, "sample": "full solves"}
    res["cfg3"] = {"note": "the reference has no mixed-precision solve; its solve of this problem is cfg1's",
                   "port_solves_per_s": port1, "c_openmp_solves_per_s": c1}

    # cfg2: Helmholtz 256x256, N=8, 1e-8 relative: per-iteration time x the GPU iteration count
    if pcg and "cfg2_helmholtz_256x256_n8" in pcg:
        iters = pcg["cfg2_helmholtz_256x256_n8"]["fp64"]["iters"]
        mo2 = O.Mesh(9, 9, E_X, E_Y, (False, False), O.sin_deform(AMP), dense_qq=True)
        M2 = O.generateMask(["D"] * 4, mo2)
        rng = np.random.default_rng(2)
        f2 = np.zeros(mo2.shape)
        for _ in range(16):
            kx, ky = rng.integers(1, 9, size=2)
            c = rng.standard_normal() / (kx ** 2 + ky ** 2)
            f2 += c * np.sin(kx * np.pi * mo2.x) * np.sin(ky * np.pi * mo2.y)
        b2 = O.gatherScatter(O.mask(O.mass(f2, mo2), M2), mo2)
        d2 = O.jacobi_diag(mo2, NU, LAM, M2)
        solve2 = port_solver(mo2, NU, LAM, M2, d2)
        t0 = time.time()
        solve2(b2, 0.0, maxiter=3)
        it_port = (time.time() - t0) / 3
        g2 = C.grid(9, E_X, E_Y, (False, False), "DDDD")
        t0 = time.time()
        C.pcg(g2, mo2.Dr, mo2.Ds, mo2.G11, mo2.G12, mo2.G22, mo2.B, b2, nu=NU, k=LAM, d=d2, tol=0.0, maxiter=20)
        it_c = (time.time() - t0) / 20
        res["cfg2_helmholtz_256x256_n8_1e-8"] = {
            "port_solves_per_s": 1.0 / (it_port * iters), "c_openmp_solves_per_s": 1.0 / (it_c * iters),
            "port_ms_per_iter": 1e3 * it_port, "c_ms_per_iter": 1e3 * it_c, "iters": iters,
            "sample": "3 (port) / 20 (C) iterations timed, times the GPU solve's iteration count"}

    # cfg4: a sample of the 512 problems (every 32nd), per-iteration time x that
    # problem's GPU iteration count, scaled to the whole batch by local DOF-iterations
    if batch and batch.get("_problems"):
        probs = batch["_problems"]
        sample = probs[::32]
        t_tot = 0.0
        work_s = 0.0
        for pb in sample:
            mo4 = O.Mesh(pb["N"] + 1, pb["N"] + 1, pb["Ex"], pb["Ey"], (False, False), O.sin_deform(0.05))
            M4 = O.generateMask(["D"] * 4, mo4)
            f4 = 2 * np.pi ** 2 * np.sin(np.pi * mo4.x) * np.sin(np.pi * mo4.y)
            b4 = O.gatherScatter(O.mask(O.mass(f4, mo4), M4), mo4)
            d4 = O.jacobi_diag(mo4, pb["nu"], pb["lam"], M4)
            g4 = C.grid(pb["N"] + 1, pb["Ex"], pb["Ey"], (False, False), "DDDD")
            t0 = time.time()
            C.pcg(g4, mo4.Dr, mo4.Ds, mo4.G11, mo4.G12, mo4.G22, mo4.B, b4, nu=pb["nu"], k=pb["lam"],
                  d=d4, tol=0.0, maxiter=10)
            t_it = (time.time() - t0) / 10
            t_tot += t_it * pb["iters"]
            work_s += mo4.x.size * pb["iters"]
        work_all = sum(pb["local"] * pb["iters"] for pb in probs)
        batch_s = t_tot * work_all / work_s
        res["cfg4_batch_512"] = {"c_openmp_solves_per_s": len(probs) / batch_s, "c_batch_s_estimate": batch_s,
                                 "sample": f"{len(sample)} of {len(probs)} problems: 10 iterations each timed, "
                                           "times the GPU iteration count, scaled by local DOF x iterations"}

    # cfg5: gradient = forward + adjoint solve on 128x128 (per-iteration time x GPU counts)
    if adjoint and adjoint.get("forward_iters"):
        mo5 = O.Mesh(9, 9, 128, 128, (False, False), O.sin_deform(0.05))
        M5 = O.generateMask(["D"] * 4, mo5)
        nu5 = np.exp(0.5 * np.sin(3 * mo5.x) * np.cos(2 * mo5.y))
        b5 = O.gatherScatter(O.mask(O.mass(np.ones(mo5.shape), mo5), M5), mo5)
        G5 = (nu5 * mo5.G11, nu5 * mo5.G12, nu5 * mo5.G22)
        d5 = O.jacobi_diag(mo5, 1.0, 0.0, M5, G=G5)
        g5 = C.grid(9, 128, 128, (False, False), "DDDD")
        t0 = time.time()
        C.pcg(g5, mo5.Dr, mo5.Ds, mo5.G11, mo5.G12, mo5.G22, mo5.B, b5, nu=1.0, k=0.0, d=d5, nug=nu5,
              tol=0.0, maxiter=20)
        t_it = (time.time() - t0) / 20
        its = adjoint["forward_iters"] + adjoint["adjoint_iters"]
        res["cfg5_gradient_128x128_n8"] = {"c_openmp_gradient_s": t_it * its, "c_ms_per_iter": 1e3 * t_it,
                                           "iters": its,
                                           "sample": "20 iterations of the variable-coefficient CG timed, times "
                                                     "the GPU forward + adjoint iteration counts"}
    return res


def cpu_time_loop(steps=20):
    """The Diffusion stepping of src/diffusion.jl:81-106 restated in NumPy
    (dense QQ', identity preconditioner, mult-weighted dots, tol 1e-8) on the
    8x8 N=8 mesh with d2d.jl's forcing: BDF3, dt = 1e-3, a bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import sem_oracle as O
    mo = O.Mesh(9, 9, 8, 8, (False, False), O.sin_deform(0.1), dense_qq=True)
    M = O.generateMask(["D"] * 4, mo)
    k, dt = 3, 1e-3
    sp = np.sin(2 * np.pi * mo.x) * np.sin(2 * np.pi * mo.y)
    u, uh, tt = sp.copy(), [np.zeros(mo.shape) for _ in range(k)], [0.0] * (k + 1)
    t0 = time.time()
    for _ in range(steps):
        uh = [u.copy()] + uh[:-1]
        tt = [tt[0]] + tt[:-1]
        tt[0] += dt
        _, bb = O.bdfExtK(tt, k)
        f = sp * (8 * np.pi ** 2 * np.cos(2 * np.pi * tt[0]) - 2 * np.pi * np.sin(2 * np.pi * tt[0]))
        rhs = O.diffusion_makeRHS(mo, 1.0, f, np.zeros(mo.shape), uh, bb, M)
        u = O.pcg(rhs, lambda v, bb=bb: O.diffusion_opLHS(v, mo, 1.0, bb[0], M), mult=mo.mult, tol=1e-8)
    el = time.time() - t0
    return {"steps_per_s": steps / el, "steps": steps, "cores": os.cpu_count(), "kind": "port",
            "sample": f"{steps} BDF3 steps of the reference-faithful NumPy restatement"}


def run_reference(args):
    step, _ = reference_apply_timer()
    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t = time.time()
        step()
        times.append(time.time() - t)
    ms = 1e3 * sum(times) / len(times)
    G = unique_dof(N_ORDER + 1, E_X, E_Y)
    val = G / (ms * 1e-3) / 1e9
    cores = os.cpu_count()
    return {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic: seeded U(-1,1) field (seed 3) on the seeded deformed mesh",
            "config": {"workload": WORKLOAD, "elements": [E_X, E_Y], "order": N_ORDER,
                       "unique_dof": G, "parallelism": "host cores (BLAS threads)"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} applies of the full workload, "
                                       "reference-faithful NumPy restatement (Julia is not "
                                       "available to run the reference itself)"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extras", action="store_true", help="skip the PCG and order-sweep extras")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--variant", type=int, default=None,
                    help="pin the FP64 operator kernel variant instead of the autotuned one")
    ap.add_argument("--extras", default="",
                    help="comma-separated subset of pcg,sweep,batch,adjoint (default: all)")
    ap.add_argument("--fd-directions", type=int, default=32,
                    help="finite-difference directions of the adjoint check (the config names 32)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)))
        return 0
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = run_ours(args, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
