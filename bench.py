#!/usr/bin/env python3
"""Benchmark: px2wav + wav2px round trips (maps/s) of real spin-0 maps at
L=1024, N=4, B=2, J_min=2, upsample=0 on McEwen-Wiaux sampling.

One step = analysis (s2let_analysis_px2wav_real) and synthesis
(s2let_synthesis_wav2px_real) of one batch of maps already resident in HBM,
through the batched device-pointer entry points of libs2let_gpu.so.

Prints one JSON line (rank 0).  Fields beyond the headline:
  e2e           same metric through the host-pointer C ABI (batch extension, the
                synthesis of one batch on a second host thread while the next
                batch's analysis runs; sequential calls and the drop-in one-map
                calls beside it), host<->device copies inside the timed region
  roofline      dominant kernel, measured live with CUDA events on its stream
  cpu_baseline  the CPU oracle (C restatement of the reference path, OpenMP) on
                the host cores, one map of the same workload
  clocks        nvidia-smi samples taken during the timed region

`--impl reference` times the reference path's CPU implementation instead (the
oracle port, all host threads) and prints the same metric.
Multi-GPU (torchrun): independent replicas, one batch per rank, max time over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
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

METRIC = "px2wav+wav2px maps/s at L=1024,N=4: mixed vs FP64 GPU at stated max err"


def max_over_ranks(x, dist=None, device="cpu"):
    """Largest x over all ranks of the process group (x itself without one):
    the time of a replica step is the slowest replica's."""
    if not dist:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank):
    """Each rank synthesises its own maps (weak scaling: distinct inputs per replica)."""
    return 1000 + rank


def whole_job_rate(units_per_rank, world, seconds):
    """Units per second over all ranks, from the slowest rank's time."""
    return world * units_per_rank / seconds


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=32,
                    help="maps per step per GPU (the split-precision contraction streams the tables once per 16 "
                         "maps; 32 lets the host-pointer path overlap copies with transforms)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="mixed: split-precision tensor-core contraction (headline; the FP64 path is timed "
                         "beside it on the same inputs); fp64: the FP64 path alone")
    ap.add_argument("--L", type=int, default=1024)
    ap.add_argument("--N", type=int, default=4)
    ap.add_argument("--B", type=float, default=2.0)
    ap.add_argument("--J_min", type=int, default=2)
    ap.add_argument("--workload", default="metric",
                    choices=["metric", "spin2", "sparsity", "uneven", "L2048", "axisym", "harmonic", "batches"],
                    help="metric: the headline (real maps, L=1024, N=4); spin2: complex spin-2 maps, "
                         "L=1024, N=5, J_min=3, error per scale; sparsity: differentiable wavelet-sparsity "
                         "loss, 32 real maps at L=256, forward + backward; uneven: 256 maps of their own L, N "
                         "and spin in one graph-replayed call against a call-per-map loop; L2048: one real map "
                         "at L=2048, N=4 with recomputed Wigner tables; axisym: axisymmetric lm and MW "
                         "transforms of one real map at L=128, J_min=0, full resolution, through the drop-in "
                         "calls (the oracle timed beside them); harmonic: lm2wav + wav2lm of one real map at "
                         "L=1024, N=4 through the drop-in calls, split precision against FP64; batches: the "
                         "metric unit at batch sizes 1, 8 and 64, split precision and FP64")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def workload(a):
    return dict(workload=f"real spin-0 maps, L={a.L}, N={a.N}, B={a.B:g}, J_min={a.J_min}, upsample=0, "
                         "MW sampling, px2wav+wav2px",
                L=a.L, N=a.N, B=a.B, J_min=a.J_min, spin=0, upsample=0, reality=1)


def power_law_real_flm(rng, L):
    """Gaussian flm with C_l ∝ (l+1)^-2, real-field symmetry, f_00 = 0."""
    l = np.repeat(np.arange(L), 2 * np.arange(L) + 1)
    m = np.concatenate([np.arange(-k, k + 1) for k in range(L)])
    amp = 1.0 / (l + 1.0)
    z = (rng.normal(size=L * L) + 1j * rng.normal(size=L * L)) * amp / np.sqrt(2.0)
    z[m == 0] = rng.normal(size=L) / (np.arange(L) + 1.0)
    neg = m < 0
    ipos = l[neg] ** 2 + l[neg] - m[neg]
    z[neg] = np.where(m[neg] % 2 == 0, 1.0, -1.0) * np.conj(z[ipos])
    z[0] = 0.0
    return z


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.dev)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# DRAM traffic / algorithmic bytes per launch of the dominant kernel, from one
# ncu capture each (DRAM bytes over the bytes the launch must move):
# profiles/fp64_contraction_L512_N4_batch8.md (traffic grows with the table
# size, so the ratio carries to the L=1024 launches) and
# profiles/ring_gamma_fused_df_L1024_N4_batch8.md (the fused ring + gamma DFT
# launches that carry most of the ring-DFT bytes: 1.437 GB of DRAM traffic for
# 1.476 GB of spectra in and gamma slices out, per bl=1024 launch of 8 maps)
TRAFFIC_RATIO = {"fp64_contraction": 1.126, "ring_dft": 0.974}


def profile_traffic(kernel, alg_bytes_per_launch):
    r = TRAFFIC_RATIO.get(kernel)
    return None if r is None else r * alg_bytes_per_launch


# timing categories of s2let_gb300/csrc/timing.h (6 and 7, the recomputed-table
# contractions and quadrature, do not run at the metric point)
KERNEL_CATS = {0: "fp64_contraction", 1: "ring_dft", 2: "gamma_dft", 3: "tiling_merge", 4: "tensor_contraction",
               5: "other", 8: "digit_slicing"}


def sht_flops(ell, s, real):
    """Direct-theta Legendre count of one spin-s SHT at band-limit ell: one
    complex x real multiply-add (4 flop) per (l, m, theta ring), ell rings."""
    ms = range(0, ell) if (real and s == 0) else range(-(ell - 1), ell)
    return 4 * ell * sum(max(0, ell - max(abs(m), abs(s))) for m in ms)


def work_flops_per_map(L, N, B, J_min):
    """Algorithmic flops of px2wav + wav2px of one real spin-0 map (multires):
    the SHT at L, the scaling SHT at B^J_min, and per scale j the SHTs of the
    directions n >= 0 kept by a real signal at bl_j = min(ceil(B^(j+1)), L)."""
    import math

    J = math.ceil(math.log(L) / math.log(B) - 1e-12)
    bl_scal = min(math.ceil(B ** J_min - 1e-12), L)
    f = sht_flops(L, 0, True) + sht_flops(bl_scal, 0, True)
    for j in range(J_min, J + 1):
        bl = min(math.ceil(B ** (j + 1) - 1e-12), L)
        Nj = min(N, bl)
        Nj += (Nj + N) % 2
        for n in range(-Nj + 1, Nj, 2):
            if n >= 0:
                f += sht_flops(bl, n, n == 0)
    return 2 * f

# bf16 MMA products per real multiply-add of the split-precision contraction
# (7 x 7 digits, the 28 with i + j <= 6)
DIGIT_PRODUCTS = 28


def measured_fma_peaks(lib):
    """FP32 and FP64 FMA throughput of this GPU, measured in this process
    (best of three launches each, about 0.1 s)."""
    out = {}
    for name, fp64, iters in (("fp32_tflops", 0, 200000), ("fp64_tflops", 1, 4000)):
        best = 0.0
        for _ in range(3):
            v = C.c_double(0.0)
            if lib.s2let_gpu_fma_rate(fp64, iters, C.byref(v)) != 0:
                raise RuntimeError("s2let_gpu_fma_rate failed")
            best = max(best, v.value)
        out[name] = best
    return out


def binding_roofline(kernels, peaks, peak_kind, fma, precision, mhz):
    """Roofline of the step's dominant kernel against the unit that binds it:
    the tensor pipe (split-precision contraction: bf16 MMA flops over the
    measured cuBLAS bf16 peak), the FP32 pipe (double-float ring DFTs: FP32
    instructions of the work model over the measured FP32 FMA instruction
    rate), the FP64 pipe (FP64 kernels: flops over the measured FP64 FMA
    peak), else HBM (algorithmic bytes over the measured copy bandwidth)."""
    dom = max(kernels, key=lambda c: kernels[c]["ms"])
    kd = kernels[dom]
    sec = kd["ms"] * 1e-3
    hbm = kd["bytes"] / sec / 1e9
    hbm_peak = peaks.get("hbm_gbs")
    if dom == "tensor_contraction":
        ach = DIGIT_PRODUCTS * kd["flops"] / sec / 1e12
        roof = {"bound": "tensor", "unit": "TFLOP/s", "achieved": ach, "peak": peaks.get("bf16_tflops"),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json bf16 burst)",
                "work": f"{DIGIT_PRODUCTS} bf16 products per FP64-equivalent multiply-add"}
    elif dom == "ring_dft" and precision == "mixed":
        ach = kd["flops"] / sec / 1e12  # the timing record carries the model FP32 instruction count
        roof = {"bound": "fp32", "unit": "Tinst/s", "achieved": ach, "peak": fma["fp32_tflops"] / 2,
                "peak_source": "measured in this run: FP32 FMA chains on every SM (s2let_gpu_fma_rate), "
                               "one instruction per FMA",
                "work": "double-float FP32 instructions of the Bluestein work model (csrc/kernels.cu ring_work)"}
    elif dom in ("fp64_contraction", "ring_dft"):
        ach = kd["flops"] / sec / 1e12
        roof = {"bound": "fp64", "unit": "TFLOP/s", "achieved": ach, "peak": fma["fp64_tflops"],
                "peak_source": "measured in this run: FP64 FMA chains on every SM (s2let_gpu_fma_rate)"}
    else:
        roof = {"bound": "hbm", "unit": "GB/s", "achieved": hbm, "peak": hbm_peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json copy)"}
    roof["frac"] = roof["achieved"] / roof["peak"] if roof["peak"] else None
    step_ms = sum(k["ms"] for k in kernels.values())
    roof.update({
        "kernel": dom, "launches_per_step": kd["launches"], "avg_launch_ms": kd["ms"] / max(kd["launches"], 1),
        "traffic": profile_traffic(dom, kd["bytes"] / max(kd["launches"], 1)),
        "share_of_step": kd["ms"] / step_ms if step_ms else None,
        "hbm": {"achieved_gbs": hbm, "peak_gbs": hbm_peak, "frac": hbm / hbm_peak if hbm_peak else None},
        "sm_mhz": mhz,
        "per_kernel_ms_per_step": {c: k["ms"] for c, k in kernels.items() if k["launches"]},
    })
    km = kernels.get("tensor_contraction")
    if km and km["launches"] and km["ms"] and dom != "tensor_contraction":
        t = DIGIT_PRODUCTS * km["flops"] / (km["ms"] * 1e-3) / 1e12
        roof["tensor_contraction"] = {"bound": "tensor", "achieved_tflops": t, "peak_tflops": peaks.get("bf16_tflops"),
                                      "frac": t / peaks.get("bf16_tflops"), "ms_per_step": km["ms"],
                                      "hbm_gbs": km["bytes"] / (km["ms"] * 1e-3) / 1e9}
    return roof


def cpu_baseline_sample(p_args, f0):
    """The oracle (C restatement of the reference path, OpenMP on all host cores):
    one map through px2wav_real + wav2px_real.  Returns (seconds, f_wav, f_scal)."""
    from oracle import oracle
    from s2let_gb300.capi import make_parameters

    port = oracle.port()
    p = make_parameters(p_args.L, p_args.B, p_args.J_min, p_args.N, 0, 0)
    t0 = time.perf_counter()
    w, s = port.px2wav(f0, p, real=True)
    port.wav2px(w, s, p, real=True)
    return time.perf_counter() - t0, w, s


def _one_map_single_thread(args):
    """Worker of the CPU throughput mode (a spawned process): one map through
    px2wav_real + wav2px_real on the oracle with one OpenMP thread.  Returns
    (px2wav seconds, wav2px seconds)."""
    L, B, J_min, N, seed = args
    os.environ["OMP_NUM_THREADS"] = "1"
    import ctypes

    from oracle import oracle
    from s2let_gb300.capi import make_parameters

    port = oracle.port()
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(1)
    except OSError:
        pass
    p = make_parameters(L, B, J_min, N, 0, 0)
    f = port.alm2map(power_law_real_flm(np.random.default_rng(seed), L), L, real=True)
    t0 = time.perf_counter()
    w, s = port.px2wav(f, p, real=True)
    t1 = time.perf_counter()
    port.wav2px(w, s, p, real=True)
    return t1 - t0, time.perf_counter() - t1


def cpu_modes(a):
    """The reference is single-threaded: one map per host core, each on one
    thread, all at once.  Throughput = cores / wall time; latency = the median
    per-process round trip (1 thread, 1 map, under the memory traffic of the
    other cores).  Processes are spawned, never forked."""
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_one_map_single_thread, [(a.L, a.B, a.J_min, a.N, 500 + k) for k in range(cores)])
    wall = time.perf_counter() - t0
    per = sorted(x + y for x, y in res)
    return {"throughput": {"value": cores / wall, "unit": "maps/s", "cores": cores, "wall_s": wall,
                           "sample": f"{cores} maps, one single-threaded process per core"},
            "latency_1thread": {"seconds_per_map": statistics.median(per),
                                "px2wav_s": statistics.median(x for x, _ in res),
                                "wav2px_s": statistics.median(y for _, y in res),
                                "value": 1.0 / statistics.median(per), "unit": "maps/s", "cores": 1}}


def run_reference(a, rank):
    if rank != 0:
        return
    rng = np.random.default_rng(0)
    from oracle import oracle

    port = oracle.port()
    from s2let_gb300.capi import make_parameters

    p = make_parameters(a.L, a.B, a.J_min, a.N, 0, 0)
    f0 = port.alm2map(power_law_real_flm(rng, a.L), a.L, real=True)
    times = []
    for i in range(a.warmup + a.steps):
        t0 = time.perf_counter()
        w, s = port.px2wav(f0, p, real=True)
        port.wav2px(w, s, p, real=True)
        if i >= a.warmup:
            times.append(time.perf_counter() - t0)
    sec = sum(times) / len(times)
    cores = os.cpu_count()
    val = 1.0 / sec
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "maps/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload(a),
        "cpu_baseline": {"value": val, "unit": "maps/s", "cores": cores, "kind": "port",
                         "sample": "one map per step (px2wav_real + wav2px_real), CPU oracle: C restatement "
                                   "of the reference S2LET layer over a restated SSHT/SO3, OpenMP on all cores"},
        "e2e": {"value": val, "unit": "maps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def spin2_flm(rng, L, s=2):
    """Spin-s Gaussian flm with C_l ∝ l^-2 for l >= |s|, zero below (no reality symmetry)."""
    l = np.repeat(np.arange(L), 2 * np.arange(L) + 1)
    amp = np.where(l >= abs(s), 1.0 / np.maximum(l, 1.0), 0.0)
    return (rng.normal(size=L * L) + 1j * rng.normal(size=L * L)) * amp / np.sqrt(2.0)


def run_workload(a, world, rank, local):
    """Secondary workloads (one JSON line each): the split-precision path against
    the FP64 path on the same inputs, CUDA-event timing after warm-up."""
    import torch

    import s2let_gb300
    from s2let_gb300 import torch_ops as T
    from s2let_gb300.capi import make_parameters

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    api = s2let_gb300.api()
    lib = api.lib
    stream = torch.cuda.current_stream(dev)

    def event_ms(fn, steps):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    rel = lambda x, y: float(((x - y).abs().max() / y.abs().max()).item())
    clocks = ClockSampler(local)
    if a.workload in ("uneven", "L2048"):
        return run_recompute_workload(a, world, rank, local)
    if a.workload in ("axisym", "harmonic"):
        return run_host_call_workload(a, world, rank)
    out = {"n_gpus": world, "steps": a.steps, "warmup": a.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "data": "synthetic"}
    if a.workload == "spin2":
        L, N, J_min, nb = 1024, 5, 3, min(a.batch, 8)
        p = make_parameters(L, 2.0, J_min, N, 2, 0)
        rng = np.random.default_rng(replica_seed(rank))
        lib.s2let_gpu_set_precision(0)
        f = torch.tensor(np.stack([api.alm2map(spin2_flm(rng, L), L, 2) for _ in range(nb)]), device=dev)
        w0, s0 = T.px2wav(f, p, precision="fp64")
        res = {}
        for prec in ("mixed", "fp64"):
            def step():
                w, sc = T.px2wav(f, p, precision=prec)
                T.wav2px(w, sc, p, precision=prec)
            for _ in range(a.warmup):
                step()
            if prec == "mixed":
                clocks.start()
            ms = max_over_ranks(event_ms(step, a.steps), None)
            if prec == "mixed":
                clk = clocks.stop()
            res[prec] = ms
        w1, s1 = T.px2wav(f, p, precision="mixed")
        r1 = T.wav2px(w1, s1, p, precision="mixed")
        J = lib.s2let_j_max(C.byref(p))
        per_scale, off = {}, 0
        for j in range(J_min, J + 1):
            n = lib.s2let_n_wav_j(j, C.byref(p))
            per_scale[str(j)] = rel(w1[:, off:off + n], w0[:, off:off + n])
            off += n
        out.update({
            "metric": "spin-2 complex px2wav+wav2px maps/s at L=1024,N=5,J_min=3 (split precision)",
            "value": whole_job_rate(nb, world, res["mixed"] * 1e-3), "unit": "maps/s",
            "ms_per_step": res["mixed"], "dtype": "bf16-split/f32-acc/f64 (complex128 I/O)",
            "config": {"workload": "complex spin-2 maps, C_l ∝ l^-2 (l >= 2), L=1024, N=5, B=2, J_min=3, "
                                   "upsample=0, MW", "batch_per_gpu": nb},
            "fp64_path": {"value": whole_job_rate(nb, world, res["fp64"] * 1e-3), "unit": "maps/s",
                          "ms_per_step": res["fp64"], "speedup_mixed_over_fp64": res["fp64"] / res["mixed"]},
            "max_rel_err_vs_fp64": {"f_wav_per_scale": per_scale, "f_scal": rel(s1, s0),
                                    "wav2px_round_trip": rel(r1, f)},
            "clocks": clk,
        })
    elif a.workload == "batches":
        # the metric unit at batch sizes 1, 8 and 64, both paths, inputs in HBM
        L = a.L
        p = make_parameters(L, a.B, a.J_min, a.N, 0, 0)
        rng = np.random.default_rng(replica_seed(rank))
        lib.s2let_gpu_set_precision(0)
        base = np.stack([api.alm2map(power_law_real_flm(rng, L), L, real=True) for _ in range(8)])
        by_batch, clk = {}, None
        for nb in (1, 8, 64):
            f = torch.tensor(np.concatenate([base] * (nb // 8 or 1))[:nb], device=dev)
            row = {}
            for prec in ("mixed", "fp64"):
                def step():
                    w, sc = T.px2wav(f, p, precision=prec)
                    T.wav2px(w, sc, p, precision=prec)
                for _ in range(a.warmup):
                    step()
                steps = a.steps if prec == "mixed" or nb <= 8 else max(1, min(a.steps, 3))
                if prec == "mixed" and nb == 64:
                    clocks.start()
                ms = max_over_ranks(event_ms(step, steps), None)
                if prec == "mixed" and nb == 64:
                    clk = clocks.stop()
                row[prec] = {"value": whole_job_rate(nb, world, ms * 1e-3), "ms_per_step": ms, "steps": steps}
            row["speedup_mixed_over_fp64"] = row["fp64"]["ms_per_step"] / row["mixed"]["ms_per_step"]
            by_batch[str(nb)] = row
            del f
            torch.cuda.empty_cache()
        out.update({
            "metric": f"px2wav+wav2px maps/s at L={L}, N={a.N} by batch size (1, 8, 64; split precision and FP64)",
            "value": by_batch["64"]["mixed"]["value"], "unit": "maps/s",
            "ms_per_step": by_batch["64"]["mixed"]["ms_per_step"], "dtype": "bf16-split/f32-acc/f64",
            "config": {"workload": f"real spin-0 maps, L={L}, N={a.N}, B={a.B:g}, J_min={a.J_min}, upsample=0, MW; "
                                   "value: batch 64, split precision; one map per call takes the double-float "
                                   "contraction, batches of more the tensor cores",
                       "l2": "f_wav of one map (34.2 M doubles at L=1024) exceeds L2"},
            "by_batch": by_batch,
            "clocks": clk,
        })
    else:
        L, nb = 256, 32
        p = make_parameters(L, 2.0, 2, 4, 0, 0)
        sz = T.sizes(p)
        g = torch.Generator().manual_seed(replica_seed(rank))
        lib.s2let_gpu_set_precision(0)
        smooth = torch.tensor(np.stack([api.alm2map(power_law_real_flm(np.random.default_rng(replica_seed(rank) + b),
                                                                         L), L, real=True) for b in range(nb)]))
        y = (smooth + 0.1 * torch.randn((nb, sz["n_px"]), generator=g, dtype=torch.float64)).to(dev)
        x0 = y.to(torch.float32)  # FP32 storage of the iterate; the transforms run on its FP64 copy
        lam, thr = 1e-3, 0.05
        grads, res = {}, {}
        for prec in ("mixed", "fp64"):
            def step():
                x = x0.to(torch.float64).requires_grad_(True)
                w, sc = T.px2wav(x, p, precision=prec)
                ws = torch.sign(w) * torch.clamp(w.abs() - thr, min=0.0)
                r = T.wav2px(ws, sc, p, precision=prec) - y
                loss = 0.5 * torch.sum(r * r) + lam * torch.sum(w.abs())
                (gx,) = torch.autograd.grad(loss, x)
                return gx
            for _ in range(a.warmup):
                grads[prec] = step()
            if prec == "mixed":
                clocks.start()
            res[prec] = event_ms(step, a.steps)
            if prec == "mixed":
                clk = clocks.stop()
        out.update({
            "metric": "wavelet-sparsity loss forward+backward maps/s, 32 real maps at L=256, N=4 (split precision)",
            "value": whole_job_rate(nb, world, res["mixed"] * 1e-3), "unit": "maps/s",
            "ms_per_step": res["mixed"], "dtype": "f32 storage, bf16-split/f32-acc/f64 transforms",
            "config": {"workload": "loss = 0.5||wav2px(soft(px2wav(x))) - y||^2 + 1e-3 ||px2wav(x)||_1, "
                                   "y = smooth Gaussian field + N(0, 0.1^2)", "L": L, "N": 4, "B": 2.0,
                       "J_min": 2, "batch_per_gpu": nb},
            "fp64_path": {"value": whole_job_rate(nb, world, res["fp64"] * 1e-3), "unit": "maps/s",
                          "ms_per_step": res["fp64"], "speedup_mixed_over_fp64": res["fp64"] / res["mixed"]},
            "max_rel_err_grad_vs_fp64": rel(grads["mixed"], grads["fp64"]),
            "clocks": clk,
        })
    if rank == 0:
        print(json.dumps(out), flush=True)


ALL_CATS = {0: "fp64_contraction", 1: "ring_dft", 2: "gamma_dft", 3: "tiling_merge", 4: "tensor_contraction",
            5: "other", 6: "recomputed_contraction", 7: "quadrature", 8: "digit_slicing"}


def step_breakdown(lib, fn, sync):
    """Milliseconds per kernel category of one call of fn (CUDA events around
    each launch, csrc/timing.h categories)."""
    lib.s2let_gpu_timing_enable(1)
    fn()
    sync()
    rep = (C.c_double * 36)()
    lib.s2let_gpu_timing_report(rep, 9)
    lib.s2let_gpu_timing_enable(0)
    return {c: round(rep[4 * i + 1], 2) for i, c in ALL_CATS.items() if rep[4 * i]}


def run_host_call_workload(a, world, rank):
    """One map through the drop-in host calls, timed on the wall clock (every
    call synchronous, host buffers, copies included)."""
    import s2let_gb300
    from oracle import oracle
    from s2let_gb300.capi import make_parameters, ptr

    api = s2let_gb300.api()
    lib = api.lib
    port = oracle.port()
    rng = np.random.default_rng(replica_seed(rank))

    def wall(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        return (time.perf_counter() - t0) / steps

    rel = lambda x, y: float(np.abs(np.asarray(x) - np.asarray(y)).max() / max(np.abs(np.asarray(y)).max(), 1e-300))
    out = {"n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "data": "synthetic", "unit": "maps/s"}
    if a.workload == "axisym":
        L = 128
        p = make_parameters(L, 2.0, 0, 1, 0, 1)
        flm = power_law_real_flm(rng, L)
        f = api.alm2map(flm, L, real=True)
        res = {}
        for name, impl in (("gpu", api), ("oracle", port)):
            def lm_round():
                fw, fs = impl.axisym_lm_analysis(flm, p)
                return fw, fs, impl.axisym_lm_synthesis(fw, fs, p)

            def mw_round():
                w_, s_ = impl.axisym("analysis", [f], p, real=True)
                return w_, s_, impl.axisym("synthesis", [w_, s_], p, real=True)

            steps = a.steps if name == "gpu" else 1
            res[name] = {"lm": (wall(lm_round, steps, 1 if name == "gpu" else 0), lm_round()),
                         "mw": (wall(mw_round, steps, 1 if name == "gpu" else 0), mw_round())}
        g, o = res["gpu"], res["oracle"]
        out.update({
            "metric": "axisymmetric lm wavelet analysis+synthesis maps/s at L=128, J_min=0, full resolution "
                      "(drop-in host calls)",
            "value": 1.0 / g["lm"][0], "ms_per_step": 1e3 * g["lm"][0], "dtype": "f64",
            "config": {"workload": "one real map, L=128, B=2, J_min=0, N=1, spin=0, upsample=1, MW, power-law flm "
                                   "(f_00 = 0); s2let_transform_axisym_lm_wav_analysis + _synthesis"},
            "max_rel_err_vs_oracle": {"f_wav_lm": rel(g["lm"][1][0], o["lm"][1][0]),
                                      "f_scal_lm": rel(g["lm"][1][1], o["lm"][1][1]),
                                      "flm": rel(g["lm"][1][2], o["lm"][1][2])},
            "round_trip_rel_err": rel(g["lm"][1][2], flm),
            "oracle_cpu": {"value": 1.0 / o["lm"][0], "unit": "maps/s", "cores": os.cpu_count(), "kind": "port"},
            "mw": {"value": 1.0 / g["mw"][0], "ms_per_step": 1e3 * g["mw"][0],
                   "api": "s2let_transform_axisym_wav_analysis_mw_real + _synthesis_mw_real",
                   "max_rel_err_vs_oracle": {"f_wav": rel(g["mw"][1][0], o["mw"][1][0]),
                                             "f": rel(g["mw"][1][2], o["mw"][1][2])},
                   "oracle_cpu_maps_per_s": 1.0 / o["mw"][0]},
        })
    else:
        L = 1024
        p = make_parameters(L, 2.0, 2, 4, 0, 0)
        flm = power_law_real_flm(rng, L)
        sz = api.sizes(p)
        res = {}
        for prec in (1, 0):
            lib.s2let_gpu_set_precision(prec)

            def round_trip():
                w_ = np.zeros(sz["n_wav"])
                s_ = np.zeros(sz["n_scal"])
                lib.s2let_analysis_lm2wav_real(ptr(w_), ptr(s_), ptr(flm), C.byref(p))
                r_ = np.zeros(L * L, np.complex128)
                lib.s2let_synthesis_wav2lm_real(ptr(r_), ptr(w_), ptr(s_), C.byref(p))
                return w_, s_, r_

            t = wall(round_trip, a.steps, 1)
            res[prec] = (t, round_trip())
        lib.s2let_gpu_set_precision(0)
        s2let_gb300.check(lib, "harmonic drop-in calls")
        out.update({
            "metric": "lm2wav+wav2lm maps/s at L=1024, N=4 (drop-in host calls, split precision)",
            "value": 1.0 / res[1][0], "ms_per_step": 1e3 * res[1][0],
            "dtype": "f64 in/out; double-float contractions and ring DFTs on the FP32 pipe (split precision)",
            "config": {"workload": "one real map's flm, L=1024, N=4, B=2, J_min=2, upsample=0; "
                                   "s2let_analysis_lm2wav_real + s2let_synthesis_wav2lm_real"},
            "fp64_path": {"value": 1.0 / res[0][0], "ms_per_step": 1e3 * res[0][0]},
            "max_rel_err_vs_fp64": {"f_wav": rel(res[1][1][0], res[0][1][0]), "flm": rel(res[1][1][2], res[0][1][2])},
            "round_trip_rel_err": rel(res[1][1][2], flm),
            "note": "one map per call streams every Wigner table of the plan once per direction (double-float "
                    "copies, 8 B per entry, two scales of a band-limit per pass; the reference API takes one map)",
        })
    if rank == 0:
        print(json.dumps(out), flush=True)


def uneven_parameters(rng, n):
    """The uneven configuration: L log-uniform on [64, 512] rounded to even,
    N uniform in {1, 3, 5}, spin uniform in {0, 2} (spin-0 maps real, spin-2
    maps complex), B = 2, J_min = 1."""
    out = []
    for _ in range(n):
        L = int(2 * round(np.exp(rng.uniform(np.log(64), np.log(512))) / 2))
        out.append((L, int(rng.choice([1, 3, 5])), int(rng.choice([0, 2]))))
    return out


def run_recompute_workload(a, world, rank, local):
    """Workloads on recomputed Wigner tables (FP64 contraction): the uneven
    batch and the L = 2048 map, whose stored tables would not fit."""
    import time

    import torch

    import s2let_gb300
    from s2let_gb300.capi import S2letParameters, make_parameters

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    api = s2let_gb300.api()
    lib = api.lib
    lib.s2let_gpu_set_precision(0)
    stream = torch.cuda.Stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    clocks = ClockSampler(local)

    def event_ms(fn, steps):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    out = {"n_gpus": world, "steps": a.steps, "warmup": a.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "data": "synthetic", "unit": "maps/s", "dtype": "f64"}
    if a.workload == "uneven":
        lib.s2let_gpu_set_table_mode(2)
        rng = np.random.default_rng(replica_seed(rank))
        maps = uneven_parameters(rng, 256)
        n = len(maps)
        params = (S2letParameters * n)()
        real = (C.c_int * n)()
        px, wav, scal, rec = [], [], [], []
        for k, (L, N, spin) in enumerate(maps):
            params[k] = make_parameters(L, 2.0, 1, N, spin, 0)
            real[k] = 1 if spin == 0 else 0
            sz = api.sizes(params[k])
            dt = torch.float64 if real[k] else torch.complex128
            flm = power_law_real_flm(rng, L) if real[k] else spin2_flm(rng, L, spin)
            f = api.alm2map(flm, L, spin, real=bool(real[k]))
            px.append(torch.from_numpy(f).to(dev))
            wav.append(torch.zeros(sz["n_wav"], dtype=dt, device=dev))
            scal.append(torch.zeros(sz["n_scal"], dtype=dt, device=dev))
            rec.append(torch.zeros_like(px[-1]))

        def arrays(idx):
            m = len(idx)
            pa = (S2letParameters * m)(*[params[k] for k in idx])
            ra = (C.c_int * m)(*[real[k] for k in idx])
            ptr = lambda ts: (C.c_void_p * m)(*[ts[k].data_ptr() for k in idx])
            return pa, ra, ptr(px), ptr(wav), ptr(scal), ptr(rec), m

        def multi_step(arr):
            pa, ra, P, W, S_, R, m = arr
            assert lib.s2let_gpu_px2wav_multi(W, S_, P, pa, ra, m, 1, sp) == 0
            assert lib.s2let_gpu_wav2px_multi(R, W, S_, pa, ra, m, 1, sp) == 0

        def loop_step():
            for k in range(n):
                p = C.byref(params[k])
                if real[k]:
                    lib.s2let_gpu_analysis_px2wav_real_batch(wav[k].data_ptr(), scal[k].data_ptr(),
                                                             px[k].data_ptr(), 1, p, sp)
                    lib.s2let_gpu_synthesis_wav2px_real_batch(rec[k].data_ptr(), wav[k].data_ptr(),
                                                              scal[k].data_ptr(), 1, p, sp)
                else:
                    lib.s2let_gpu_analysis_px2wav_batch(wav[k].data_ptr(), scal[k].data_ptr(),
                                                        px[k].data_ptr(), 1, p, sp)
                    lib.s2let_gpu_synthesis_wav2px_batch(rec[k].data_ptr(), wav[k].data_ptr(),
                                                         scal[k].data_ptr(), 1, p, sp)

        allidx = list(range(n))
        arr = arrays(allidx)
        t0 = time.time()
        multi_step(arr)  # builds every plan (eager pass)
        torch.cuda.synchronize()
        build_s = time.time() - t0
        for _ in range(max(a.warmup, 2)):  # the second call captures the graph
            multi_step(arr)
        clocks.start()
        ms = event_ms(lambda: multi_step(arr), a.steps)
        clk = clocks.stop()
        err = max(float(((rec[k] - px[k]).abs().max() / px[k].abs().max()).item()) for k in range(n))
        for _ in range(a.warmup):
            loop_step()
        loop_ms = event_ms(loop_step, a.steps)
        # FP32 storage: the same maps in single precision through the multi-map
        # _f32 calls (widened to FP64 scratch inside the graph, rounded back)
        px32 = [t.to(torch.float32 if real[k] else torch.complex64) for k, t in enumerate(px)]
        wav32 = [t.to(torch.float32 if real[k] else torch.complex64) for k, t in enumerate(wav)]
        scal32 = [t.to(torch.float32 if real[k] else torch.complex64) for k, t in enumerate(scal)]
        rec32 = [torch.zeros_like(t) for t in px32]
        ptr32 = lambda ts: (C.c_void_p * n)(*[t.data_ptr() for t in ts])
        P32, W32, S32, R32 = ptr32(px32), ptr32(wav32), ptr32(scal32), ptr32(rec32)
        pa_all, ra_all = arr[0], arr[1]

        def multi_step_f32():
            assert lib.s2let_gpu_px2wav_multi_f32(W32, S32, P32, pa_all, ra_all, n, 1, sp) == 0
            assert lib.s2let_gpu_wav2px_multi_f32(R32, W32, S32, pa_all, ra_all, n, 1, sp) == 0

        for _ in range(max(a.warmup, 2)):
            multi_step_f32()
        ms32 = event_ms(multi_step_f32, a.steps)
        err32 = max(float(((rec32[k].to(rec[k].dtype) - rec[k]).abs().max() / rec[k].abs().max()).item())
                    for k in range(n))
        # configuration 4 as specified: FP32 storage, split precision (double-float
        # contractions on the recomputed tables), autotuned launch shapes, graph-replayed
        lib.s2let_gpu_set_precision(1)
        for _ in range(max(a.warmup, 2)):
            multi_step_f32()
        ms32_mx = event_ms(multi_step_f32, a.steps)
        rec32_mx = [r.clone() for r in rec32]
        err32_mx = max(float(((rec32_mx[k].to(rec[k].dtype) - rec[k]).abs().max() / rec[k].abs().max()).item())
                       for k in range(n))
        for _ in range(max(a.warmup, 2)):
            multi_step(arr)
        ms_mx = event_ms(lambda: multi_step(arr), a.steps)
        err_mx = max(float(((rec[k] - px[k]).abs().max() / px[k].abs().max()).item()) for k in range(n))
        for _ in range(a.warmup):
            loop_step()
        loop_mx_ms = event_ms(loop_step, a.steps)
        lib.s2let_gpu_set_precision(0)
        # autotuned launch shapes (tuned on the first call of each shape, cache in a temporary file)
        import tempfile

        tune_dir = tempfile.mkdtemp(prefix="s2let_tune_")
        os.environ["S2LET_GPU_AUTOTUNE_CACHE"] = os.path.join(tune_dir, "autotune.txt")
        old_tune = lib.s2let_gpu_autotune(1)
        t0 = time.time()
        for _ in range(max(a.warmup, 2) + 1):  # tuning pass, graph capture, a replay
            multi_step(arr)
        torch.cuda.synchronize()
        tune_s = time.time() - t0
        ms_tuned = event_ms(lambda: multi_step(arr), a.steps)
        # the configuration-4 recipe with the tuned shapes (tuning again at split precision)
        lib.s2let_gpu_set_precision(1)
        for _ in range(max(a.warmup, 2) + 1):
            multi_step_f32()
        torch.cuda.synchronize()
        ms_cfg4 = event_ms(multi_step_f32, a.steps)
        bd_cfg4 = step_breakdown(lib, multi_step_f32, torch.cuda.synchronize)  # eager while timing
        lib.s2let_gpu_set_precision(0)
        ntuned = lib.s2let_gpu_autotune_entries((C.c_int * 5000)(), (C.c_double * 2000)(), 1000)
        lib.s2let_gpu_autotune(old_tune)
        buckets = {}
        for lo, hi in ((64, 128), (128, 256), (256, 513)):
            idx = [k for k in range(n) if lo <= maps[k][0] < hi]
            if not idx:
                continue
            arr_b = arrays(idx)
            for _ in range(3):
                multi_step(arr_b)
            bms = event_ms(lambda: multi_step(arr_b), a.steps)
            buckets[f"L{lo}-{min(hi, 512)}"] = {"maps": len(idx), "maps_per_s": len(idx) / (bms * 1e-3),
                                                "ms": bms}
        out.update({
            "metric": "uneven batch px2wav+wav2px maps/s (256 maps, own L/N/spin each, one graph-replayed call; "
                      "FP32 storage, split precision, autotuned launch shapes)",
            "value": whole_job_rate(n, world, ms_cfg4 * 1e-3), "ms_per_step": ms_cfg4,
            "per_kernel_ms_per_step": bd_cfg4,
            "dtype": "f32 storage; double-float recomputed-table contractions and ring DFTs (split precision)",
            "config": {"workload": "256 maps, L log-uniform on [64, 512] rounded to even, N in {1,3,5}, "
                                   "spin in {0,2} (spin 0 real, spin 2 complex), B=2, J_min=1, MW, "
                                   "power-law flm; recomputed Wigner tables",
                       "distinct_parameter_sets": len({(m[0], m[1], m[2]) for m in maps}),
                       "l2": "inputs and outputs of the 256 maps exceed L2"},
            "fp64": {"value": whole_job_rate(n, world, ms * 1e-3), "ms_per_step": ms,
                     "what": "FP64 storage, FP64 contractions, graph-replayed"},
            "split_precision": {"value": whole_job_rate(n, world, ms_mx * 1e-3), "ms_per_step": ms_mx,
                                "what": "FP64 storage, split precision, graph-replayed",
                                "max_rel_err_round_trip": err_mx},
            "split_precision_fp32_storage": {"value": whole_job_rate(n, world, ms32_mx * 1e-3),
                                             "ms_per_step": ms32_mx,
                                             "max_rel_err_vs_fp64": err32_mx},
            "one_call_per_map_loop": {"value": whole_job_rate(n, world, loop_ms * 1e-3), "ms_per_step": loop_ms,
                                      "what": "FP64, one s2let_gpu_*_batch call per map"},
            "one_call_per_map_loop_split": {"value": whole_job_rate(n, world, loop_mx_ms * 1e-3),
                                            "ms_per_step": loop_mx_ms,
                                            "what": "split precision, one call per map"},
            "fp32_storage": {"value": whole_job_rate(n, world, ms32 * 1e-3), "ms_per_step": ms32,
                             "api": "s2let_gpu_px2wav_multi_f32 + s2let_gpu_wav2px_multi_f32 (graph-replayed)",
                             "max_rel_err_vs_fp64_storage": err32},
            "autotuned": {"value": whole_job_rate(n, world, ms_tuned * 1e-3), "ms_per_step": ms_tuned,
                          "what": "FP64, tuned launch shapes", "tuning_s": tune_s, "shapes_recorded": ntuned},
            "per_L_bucket": buckets,
            "plan_build_s": build_s,
            "max_rel_err_round_trip": err,
            "clocks": clk,
        })
    else:
        L = 2048
        p = make_parameters(L, 2.0, 2, 4, 0, 0)
        rng = np.random.default_rng(replica_seed(rank))
        lib.s2let_gpu_set_table_mode(2)
        f = torch.from_numpy(api.sht(1, power_law_real_flm(rng, L), L, 0, True)).to(dev)[None, :].contiguous()
        lib.s2let_gpu_set_table_mode(0)
        sz = api.sizes(p)
        w = torch.zeros((1, sz["n_wav"]), dtype=torch.float64, device=dev)
        s_ = torch.zeros((1, sz["n_scal"]), dtype=torch.float64, device=dev)
        r = torch.zeros_like(f)
        pp = C.byref(p)

        def step():
            lib.s2let_gpu_analysis_px2wav_real_batch(w.data_ptr(), s_.data_ptr(), f.data_ptr(), 1, pp, sp)
            lib.s2let_gpu_synthesis_wav2px_real_batch(r.data_ptr(), w.data_ptr(), s_.data_ptr(), 1, pp, sp)

        t0 = time.time()
        step()
        torch.cuda.synchronize()
        build_s = time.time() - t0
        for _ in range(max(1, a.warmup - 1)):
            step()
        ms64 = event_ms(step, a.steps)
        bd64 = step_breakdown(lib, step, torch.cuda.synchronize)
        err64 = float(((r - f).abs().max() / f.abs().max()).item())
        w64 = w.clone()
        lib.s2let_gpu_set_precision(1)  # split precision: double-float recomputed-table contractions
        for _ in range(max(1, a.warmup - 1)):
            step()
        clocks.start()
        ms = event_ms(step, a.steps)
        clk = clocks.stop()
        bd = step_breakdown(lib, step, torch.cuda.synchronize)
        lib.s2let_gpu_set_precision(0)
        out.update({
            "metric": "px2wav+wav2px maps/s at L=2048, N=4 (recomputed Wigner tables, split precision)",
            "per_kernel_ms_per_step": bd,
            "value": whole_job_rate(1, world, ms * 1e-3), "ms_per_step": ms,
            "dtype": "double-float recomputed-table contractions and ring DFTs, FP64 quadrature",
            "fp64_path": {"value": whole_job_rate(1, world, ms64 * 1e-3), "ms_per_step": ms64,
                          "max_rel_err_round_trip": err64, "per_kernel_ms_per_step": bd64},
            "max_rel_err_f_wav_vs_fp64": float(((w - w64).abs().max() / w64.abs().max()).item()),
            "config": {"workload": "one real spin-0 map, L=2048, N=4, B=2, J_min=2, upsample=0, MW, "
                                   "power-law band-limited flm", "table_bytes_device": lib.s2let_gpu_plan_bytes()},
            "plan_build_s": build_s,
            "max_rel_err_round_trip": float(((r - f).abs().max() / f.abs().max()).item()),
            "clocks": clk,
        })
    lib.s2let_gpu_set_table_mode(0)
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    a = args_()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank)
        return
    if a.workload != "metric":
        run_workload(a, world, rank, local)
        return

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import s2let_gb300
    from s2let_gb300.capi import make_parameters

    api = s2let_gb300.api()
    lib = api.lib
    lib.s2let_gpu_set_precision(0)  # inputs are synthesised on the FP64 path
    p = make_parameters(a.L, a.B, a.J_min, a.N, 0, 0)
    sz = api.sizes(p)
    nb = a.batch
    npx, nw, ns = sz["n_px"], sz["n_wav"], sz["n_scal"]

    # seeded band-limited inputs, synthesised on the GPU from power-law flm
    rng = np.random.default_rng(replica_seed(rank))
    f_host = np.stack([api.alm2map(power_law_real_flm(rng, a.L), a.L, real=True) for _ in range(nb)])
    s2let_gb300.check(lib, "alm2map_real")
    f = torch.tensor(f_host, device=dev)
    lib.s2let_gpu_set_precision(1 if a.precision == "mixed" else 0)
    w = torch.zeros((nb, nw), dtype=torch.float64, device=dev)
    sc = torch.zeros((nb, ns), dtype=torch.float64, device=dev)
    fr = torch.zeros_like(f)
    stream = torch.cuda.current_stream(dev)
    st = C.c_void_p(stream.cuda_stream)
    vp = lambda t: C.c_void_p(t.data_ptr())

    def step():
        rc = lib.s2let_gpu_analysis_px2wav_real_batch(vp(w), vp(sc), vp(f), nb, C.byref(p), st)
        rc |= lib.s2let_gpu_synthesis_wav2px_real_batch(vp(fr), vp(w), vp(sc), nb, C.byref(p), st)
        if rc:
            raise RuntimeError(lib.s2let_gpu_last_error_string().decode())

    t0 = time.perf_counter()
    step()  # builds the plan (Wigner tables, FFT data)
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - t0
    for _ in range(max(a.warmup - 1, 0)):
        step()
    torch.cuda.synchronize()

    def timed(nsteps):
        """Device time of nsteps steps (CUDA events on the launching stream), max over ranks."""
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(nsteps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return max_over_ranks(e0.elapsed_time(e1) / nsteps, dist, dev)

    # ---- timed region (device-resident inputs) ----
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lib.s2let_gpu_launch_count()
    ms_max = timed(a.steps)
    launches = lib.s2let_gpu_launch_count() - launches0
    clk = clocks.stop()
    value = whole_job_rate(nb, world, ms_max * 1e-3)
    fault = lib.s2let_gpu_device_fault()
    if fault:
        raise RuntimeError(f"device fault flag {fault} raised by the split-precision contraction")

    # round-trip fidelity on the band-limited inputs
    rt_err = float(((fr - f).abs().max() / f.abs().max()).item())

    # ---- the FP64 path on the same inputs: speed and the error of the mixed outputs ----
    fp64 = None
    if a.precision == "mixed":
        w_mx, sc_mx, fr_mx = w.clone(), sc.clone(), fr.clone()
        lib.s2let_gpu_set_precision(0)
        for _ in range(a.warmup):
            step()
        ms64 = timed(a.steps)
        rel = lambda x, y: float(((x - y).abs().max() / y.abs().max()).item())
        fp64 = {"value": whole_job_rate(nb, world, ms64 * 1e-3), "unit": "maps/s", "ms_per_step": ms64,
                "speedup_mixed_over_fp64": ms64 / ms_max,
                "max_rel_err_mixed_vs_fp64": {"f_wav": rel(w_mx, w), "f_scal": rel(sc_mx, sc),
                                              "wav2px": rel(fr_mx, fr)}}
        w.copy_(w_mx)
        sc.copy_(sc_mx)
        fr.copy_(fr_mx)
        lib.s2let_gpu_set_precision(1)

    # ---- roofline: one instrumented step, CUDA events around each launch ----
    peaks, peak_kind = measured_peaks()
    fma = measured_fma_peaks(lib)

    def instrumented_step():
        lib.s2let_gpu_timing_enable(1)
        step()
        torch.cuda.synchronize()
        rep = (C.c_double * 36)()
        lib.s2let_gpu_timing_report(rep, 9)
        lib.s2let_gpu_timing_enable(0)
        return {c: {"launches": int(rep[4 * i]), "ms": rep[4 * i + 1], "flops": rep[4 * i + 2],
                    "bytes": rep[4 * i + 3]} for i, c in KERNEL_CATS.items()}

    kernels = instrumented_step()
    mhz = (clk or {}).get("sm_mhz")
    roof = binding_roofline(kernels, peaks, peak_kind, fma, a.precision, mhz)
    if fp64 is not None:
        # the FP64 path on the same inputs: its step breakdown and roofline
        lib.s2let_gpu_set_precision(0)
        k64 = instrumented_step()
        lib.s2let_gpu_set_precision(1)
        wpm = work_flops_per_map(a.L, a.N, a.B, a.J_min)
        f64_flops = wpm * nb  # algorithmic flops of one step
        t64 = f64_flops / (fp64["ms_per_step"] * 1e-3) / 1e12
        fp64["roofline"] = {
            "bound": "fp64", "unit": "TFLOP/s", "achieved": t64, "peak": fma["fp64_tflops"],
            "frac": t64 / fma["fp64_tflops"],
            "peak_source": "measured in this run: FP64 FMA chains on every SM (s2let_gpu_fma_rate)",
            "work": f"{wpm:.4g} flop per map (direct-theta Legendre count, both directions)",
            "per_kernel_ms_per_step": {c: k["ms"] for c, k in k64.items() if k["launches"]},
            "dominant_kernel": binding_roofline(k64, peaks, peak_kind, fma, "fp64", mhz),
        }

    # ---- e2e through the host-pointer C ABI ----
    # The timed region holds every host <-> device copy: the maps in, the
    # wavelet and scaling coefficients out and back in (analysis and synthesis
    # are separate calls with host buffers, as a C caller makes them), the
    # reconstructed maps out.  Primary: the host-pointer batch extension (all
    # maps of the step in one call per direction).  Beside it: the drop-in
    # one-map functions, one call per map.
    e2e = None
    if not a.no_e2e:
        fh = torch.empty((nb, npx), dtype=torch.float64, pin_memory=True)
        fh.copy_(torch.tensor(f_host))
        wh = torch.empty((nb, nw), dtype=torch.float64, pin_memory=True)
        sh = torch.empty((nb, ns), dtype=torch.float64, pin_memory=True)
        frh = torch.empty((nb, npx), dtype=torch.float64, pin_memory=True)

        calls = []  # per call: wall ms and the copy trace (CUDA events on the copying streams)
        trace = (C.c_double * 10)()

        def traced_call(name, fn, *args):
            lib.s2let_gpu_copy_trace_enable(1)
            t0 = time.perf_counter()
            fn(*args)
            ms = 1e3 * (time.perf_counter() - t0)
            lib.s2let_gpu_copy_trace_report(trace)
            rec = {"call": name, "ms": round(ms, 2)}
            for d, tag in ((0, "h2d"), (1, "d2h")):
                gb, busy, span = trace[5 * d + 1] / 1e9, trace[5 * d + 2], trace[5 * d + 3]
                rec[tag] = {"GB": round(gb, 3), "span_ms": round(span, 2),
                            "GBps": round(gb / span * 1e3, 1) if span > 0 else None,
                            "copies": int(trace[5 * d]), "by_kernel": int(trace[5 * d + 4])}
            calls.append(rec)

        def e2e_batch_step():
            traced_call("analysis", lib.s2let_gpu_analysis_px2wav_real_host_batch, vp(wh), vp(sh), vp(fh), nb,
                        C.byref(p))
            traced_call("synthesis", lib.s2let_gpu_synthesis_wav2px_real_host_batch, vp(frh), vp(wh), vp(sh), nb,
                        C.byref(p))
            s2let_gb300.check(lib, "host batch API")

        def e2e_single_step():
            for b in range(nb):
                lib.s2let_analysis_px2wav_real(vp(wh[b]), vp(sh[b]), vp(fh[b]), C.byref(p))
                lib.s2let_synthesis_wav2px_real(vp(frh[b]), vp(wh[b]), vp(sh[b]), C.byref(p))
            s2let_gb300.check(lib, "host API")

        def e2e_single_same_step():  # one map's host buffers, reused by every call
            for _ in range(nb):
                lib.s2let_analysis_px2wav_real(vp(wh[0]), vp(sh[0]), vp(fh[0]), C.byref(p))
                lib.s2let_synthesis_wav2px_real(vp(frh[0]), vp(wh[0]), vp(sh[0]), C.byref(p))
            s2let_gb300.check(lib, "host API")

        step_ms = []

        def host_rate(fn, steps, record=False, warmup=1):
            for _ in range(warmup):
                fn()
            if dist:
                dist.barrier()
            t0 = time.perf_counter()
            for _ in range(steps):
                t1 = time.perf_counter()
                fn()
                if record:
                    step_ms.append(1e3 * (time.perf_counter() - t1))
            return max_over_ranks((time.perf_counter() - t0) / steps, dist, dev)

        # Pipelined calls: the synthesis of batch k runs on a second host thread
        # while this thread runs the analysis of batch k+1 (two sets of host
        # f_wav / f_scal buffers, alternating).  Each call keeps its own CUDA
        # streams, so the two calls' transforms share the GPU and their f_wav
        # copies use the two directions of the link at the same time.  The
        # timed region holds every call of `steps` round trips, pipeline fill
        # and drain included: the first analysis and the last synthesis run
        # alone.  The result maps of every synthesis go to host memory.
        wh2 = [wh, torch.empty((nb, nw), dtype=torch.float64, pin_memory=True)]
        sh2 = [sh, torch.empty((nb, ns), dtype=torch.float64, pin_memory=True)]
        prec = 1 if a.precision == "mixed" else 0
        import concurrent.futures as cf

        def synth_thread_init():
            torch.cuda.set_device(local)
            lib.s2let_gpu_set_precision(prec)  # per-thread setting

        pool = cf.ThreadPoolExecutor(max_workers=1, initializer=synth_thread_init)
        pipe_calls = []

        def synth_call(k):
            t0 = time.perf_counter()
            rc = lib.s2let_gpu_synthesis_wav2px_real_host_batch(vp(frh), vp(wh2[k % 2]), vp(sh2[k % 2]), nb,
                                                                C.byref(p))
            pipe_calls.append(("synthesis", k, t0, time.perf_counter()))
            if rc:
                raise RuntimeError(lib.s2let_gpu_last_error_string().decode())

        def pipelined(steps):
            fut = None
            for k in range(steps + 1):
                if k >= 1:
                    fut = pool.submit(synth_call, k - 1)
                if k < steps:
                    t0 = time.perf_counter()
                    rc = lib.s2let_gpu_analysis_px2wav_real_host_batch(vp(wh2[k % 2]), vp(sh2[k % 2]), vp(fh), nb,
                                                                       C.byref(p))
                    pipe_calls.append(("analysis", k, t0, time.perf_counter()))
                    if rc:
                        raise RuntimeError(lib.s2let_gpu_last_error_string().decode())
                if fut is not None:
                    fut.result()
                    fut = None

        # clocks sampled over the e2e steps as over the device-timed region
        # (GPU-idle gaps between copy-bound phases make P-state behaviour matter here)
        e2e_clocks = ClockSampler(local)
        e2e_clocks.start()
        e2e_s = host_rate(e2e_batch_step, a.steps, record=True, warmup=max(1, a.warmup))
        e2e_clk = e2e_clocks.stop()
        lib.s2let_gpu_copy_trace_enable(0)
        timed_calls = calls[-2 * a.steps:]
        seq_rt = float((frh - fh).abs().max() / fh.abs().max())
        pipelined(2)  # warm-up: the second thread's streams, both host buffer sets, two calls at once
        frh.zero_()
        pipe_calls.clear()
        pipe_clocks = ClockSampler(local)
        pipe_clocks.start()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        pipelined(a.steps)
        pipe_s = max_over_ranks((time.perf_counter() - t0) / a.steps, dist, dev)
        pipe_clk = pipe_clocks.stop()
        pool.shutdown()
        pipe_rt = float((frh - fh).abs().max() / fh.abs().max())
        tp0 = min(c[2] for c in pipe_calls)
        pipe_trace = [{"call": c[0], "batch": c[1], "start_ms": round(1e3 * (c[2] - tp0), 1),
                       "ms": round(1e3 * (c[3] - c[2]), 1)} for c in sorted(pipe_calls, key=lambda c: c[2])]

        def call_stats(name):
            cs = [c for c in timed_calls if c["call"] == name]
            big = "d2h" if name == "analysis" else "h2d"  # the f_wav direction of the call
            return {"median_ms": statistics.median(c["ms"] for c in cs),
                    "min_ms": min(c["ms"] for c in cs), "max_ms": max(c["ms"] for c in cs),
                    f"f_wav_{big}_GBps_median": statistics.median(c[big]["GBps"] for c in cs),
                    f"f_wav_{big}_GBps_min": min(c[big]["GBps"] for c in cs)}
        single_s = host_rate(e2e_single_step, max(1, min(a.steps, 2)))
        single_same_s = host_rate(e2e_single_same_step, 1)
        e2e = {"value": whole_job_rate(nb, world, pipe_s), "unit": "maps/s",
               "h2d_bytes_per_step": nb * (npx + nw + ns) * 8, "d2h_bytes_per_step": nb * (nw + ns + npx) * 8,
               "api": "s2let_gpu_analysis_px2wav_real_host_batch + s2let_gpu_synthesis_wav2px_real_host_batch "
                      f"({nb} maps per call, pinned host buffers); synthesis of batch k on a second host thread "
                      "while the analysis of batch k+1 runs",
               "timed": f"{a.steps} round trips of {nb} maps, pipeline fill and drain included",
               "max_rel_err_round_trip": pipe_rt,
               "calls": pipe_trace,
               "clocks": pipe_clk,
               "sequential_calls": {
                   "value": whole_job_rate(nb, world, e2e_s), "unit": "maps/s",
                   "what": "analysis then synthesis, one call at a time",
                   "max_rel_err_round_trip": seq_rt,
                   "step_ms": [round(x, 1) for x in step_ms],
                   "per_call": {"analysis": call_stats("analysis"), "synthesis": call_stats("synthesis")},
                   "copy_trace": timed_calls,
                   "clocks": e2e_clk,
                   "median_step_value": whole_job_rate(nb, world, statistics.median(step_ms) / 1e3)
                   if step_ms else None},
               "dropin_one_map_per_call": {"value": whole_job_rate(nb, world, single_s), "unit": "maps/s",
                                           "api": "s2let_analysis_px2wav_real + s2let_synthesis_wav2px_real",
                                           "what": f"one call per map over the {nb} maps' page-locked host buffers"},
               "dropin_one_map_same_buffers": {"value": whole_job_rate(nb, world, single_same_s), "unit": "maps/s",
                                               "what": f"the same calls {nb} times on one map's host buffers"}}

    # ---- CPU baseline (rank 0, N=1) and the error against it ----
    cpu = None
    err_vs_oracle = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        sec, w_o, s_o = cpu_baseline_sample(a, f_host[0])
        modes = cpu_modes(a)
        thr = modes["throughput"]
        cpu = {"value": thr["value"], "unit": "maps/s", "cores": thr["cores"], "kind": "port",
               "sample": f"{thr['cores']} maps of the same workload (px2wav_real + wav2px_real), one "
                         f"single-threaded process per host core, {thr['wall_s']:.1f} s wall; CPU oracle = C "
                         "restatement of the reference S2LET layer over restated SSHT/SO3 (the reference is "
                         "single-threaded)",
               "latency_1thread": modes["latency_1thread"],
               "openmp_one_map": {"value": 1.0 / sec, "unit": "maps/s", "cores": os.cpu_count(),
                                  "sample": f"1 map, the oracle's OpenMP loops on all cores, {sec:.1f} s"}}
        wg = w[0].cpu().numpy()
        sg = sc[0].cpu().numpy()
        err_vs_oracle = max(float(np.abs(wg - w_o).max() / np.abs(w_o).max()),
                            float(np.abs(sg - s_o).max() / np.abs(s_o).max()))

    if rank != 0:
        return
    cfg = workload(a)
    cfg.update({"batch_per_gpu": nb, "precision": a.precision, "parallelism": f"replicas x{world}",
                "l2_policy": f"inputs larger than L2 (129 MB): f {npx * 8 / 1e6:.1f} MB + f_wav {nw * 8 / 1e6:.0f} MB "
                             f"per map x {nb} maps, no flush needed",
                "plan_build_s": plan_s})
    out = {
        "metric": METRIC, "value": value, "unit": "maps/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if a.precision == "fp64" else "bf16-split/f32-acc/f64",
        "data": "synthetic: Gaussian flm, C_l ∝ (l+1)^-2, real-field symmetry, seeded; maps by GPU alm2map",
        "config": cfg, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        "gpu_launches": launches, "fp64_path": fp64,
        "max_rel_err_vs_oracle": err_vs_oracle, "roundtrip_rel_err": rt_err,
    }
    print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
