"""Benchmark of the cell-model update on GB300 (one JSON line on stdout).

Workload (default): the precision form -- 4,194,304 ten Tusscher 2006 epicardial cells (a
2048 x 2048 sheet, reaction step only), FP32 gates/currents with compensated FP32 accumulators, per-cell
g_Na/g_Kr/g_K1 scaled by seeded U[0.9, 1.1], stimulus -52 pA/pF for 1 ms every 800 ms,
dt = 0.01 ms. One step = one dt update of every cell. Inputs are synthetic (seeded), and the
cell state (~430 MB) is larger than L2, so no flush is needed between steps.

value     cell-steps/s, state resident in HBM, the fused driver step (cm_batch_run)
e2e       the same through the drop-in C ABI with pinned HOST Vm/i_ext: cm_batch_step_update
          copies Vm and i_ext in and Vm out every step (acCELLerate's CalcCellModels + Godunov)
plain_fp64  the plain FP64 kernel on the same workload (the reference's arithmetic)
roofline  the dominant kernel (the autotuned precision-form shape) against the measured HBM copy
cpu_baseline  the oracle (C restatement of the reference Calc) on the host cores, bounded sample

--impl reference runs the reference's CPU implementation of the path (the oracle port of its
Calc; the reference itself cannot be built where its sources are absent) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_CELLS = 2048 * 2048
DT = 1e-5
BCL = 0.8
METRIC = "cell-steps/s on 1 GB300: surrogate+FP32 vs plain FP64 at <=1 ms APD90 error"
UNIT = "cell-steps/s"
# Algorithmic bytes per cell-step of the precision-form kernel: 15 FP32 states plus the
# CaSR/Na_i/K_i compensated pairs (2 x FP32 each) read and written (168 B), the Vm hi/lo
# pair read and written (16 B), 3 FP32 per-cell conductances read (12 B).
MIXED_BYTES_PER_CELL_STEP = 2 * (15 * 4 + 3 * 8) + 2 * 8 + 3 * 4
# Launch shapes of cm_batch_set_launch (variant index -> kernel); 5 and 6 are bulk-copy staged.
MIXED_KERNELS = ["tt2_mixed_kernel<256>", "tt2_mixed_kernel<128>", "tt2_mixed_kernel<256,3>",
                 "tt2_mixed_kernel<512>", "tt2_mixed_kernel<64>", "mixed_staged_kernel<5,256>",
                 "mixed_staged_kernel<5,128>"]
# dram__bytes_read.sum + dram__bytes_write.sum of one launch, from the ncu capture summarised in
# profiles/mixed_staged_tt2_4M_cells.md (same workload, launch shape 6, grid mode 4).
MEASURED_TRAFFIC = {"mixed_staged_kernel<5,128>": 436_239_360 + 327_127_808}
# tt2_fp64_kernel: 18 FP64 states r+w (288 B), Vm r+w (16 B), 3 FP64 conductances (24 B).
FP64_BYTES_PER_CELL_STEP = 2 * 18 * 8 + 2 * 8 + 3 * 8
WORKLOAD = "tt2006-epi-precision-form-2048x2048"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.out = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_batch(cm, precision, stream, n=N_CELLS, seed=2):
    from cardiomechanics_gb300 import workloads as W
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    b = cm.Batch(p, n, precision, stream=stream)
    sc = W.conductance_scales(seed, n, 3, 0.9, 1.1)
    for k, name in enumerate(W.TT2_HETERO):
        b.add_hetero_value(name, p.get(name) * sc[k])
    return p, b


def time_device_steps(torch, cm, b, stream, vm, steps, warmup, t0):
    """K fused driver steps on the batch's stream, timed with events on that stream."""
    from cardiomechanics_gb300 import workloads as W
    kw = dict(textbegin=0.0, textlen=1e-3, bcl=BCL, amplitude=W.TT2_STIM_NA)
    b.run(vm, warmup, t0=t0, **kw)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    b.run(vm, steps, t0=t0 + warmup * DT, **kw)
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3


class CPUSample:
    """The oracle (C restatement of the reference Calc) on a bounded sample of the workload:
    the first `cells` cells, advanced `steps` time steps per call, all host threads."""

    def __init__(self, cells=4096, threads=None):
        import oracle as O
        from cardiomechanics_gb300 import workloads as W
        self.O, self.W = O, W
        self.port = O.Port()
        self.threads = threads or os.cpu_count() or 1
        self.cells = cells
        self.P = self.port.param_vector(O.TT2, O.load_params(O.TT2))
        self.T = self.port.tables(O.TT2, self.P, DT)
        sc = W.conductance_scales(2, N_CELLS, 3, 0.9, 1.1, cells=np.arange(cells))
        names = self.port.param_names(O.TT2)
        self.het = {k: self.P[names.index(k)] * sc[i] for i, k in enumerate(W.TT2_HETERO)}
        self.B = self.port.init_state(O.TT2, self.P, cells)
        self.vm = np.full(cells, self.port.init_vm(O.TT2, self.P))
        self.t = 0.0

    def advance(self, steps):
        """Advance the sample; returns elapsed seconds."""
        t0 = time.perf_counter()
        self.port.run(self.O.TT2, self.P, self.T, self.B, self.vm, steps, DT, t0=self.t, textbegin=0.0,
                      textlen=1e-3, bcl=BCL, amp=self.W.TT2_STIM_NA, het=self.het, n_threads=self.threads)
        self.t += steps * DT
        return time.perf_counter() - t0

    def describe(self, steps, seconds):
        return {"unit": UNIT, "cores": self.threads, "kind": "port",
                "sample": f"first {self.cells} of the {N_CELLS} cells x {steps} steps (oracle C restatement "
                          f"of the reference Calc, {self.threads} threads, {seconds:.1f} s)"}


def cpu_baseline(seconds=10.0, cells=4096):
    """Oracle throughput on the host cores over about `seconds` of work; cell-steps/s."""
    smp = CPUSample(cells)
    done, el = 0, 0.0
    while el < seconds:
        el += smp.advance(500)
        done += 500
    d = smp.describe(done, el)
    d["value"] = cells * done / el
    return d


def run_reference(args):
    """The reference arm: the reference's CPU path (the oracle port of its Calc; the reference
    sources are not on the GPU host) on all host cores. Each step advances the cell sample by a
    chunk sized so that warmup + steps take about a minute and a half in total."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle as O
    O.build_port()
    smp = CPUSample(4096)
    rate = smp.cells * 200 / smp.advance(200)  # calibration
    total = args.steps + args.warmup
    chunk = int(max(1, min(5000, rate * 90.0 / max(1, total) / smp.cells)))
    for _ in range(args.warmup):
        smp.advance(chunk)
    times = [smp.advance(chunk) for _ in range(args.steps)]
    v = float(np.median([smp.cells * chunk / t for t in times]))
    cb = smp.describe(chunk * args.steps, float(sum(times)))
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * N_CELLS / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": N_CELLS, "dt_ms": DT * 1e3, "bcl_ms": BCL * 1e3,
                       "note": f"CPU: each step advances a {smp.cells}-cell sample {chunk} time steps"},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


SUR_CELLS = 1 << 20
SUR_BCL = 0.5
SUR_SUBSTEPS = 10


def advance_protocol(t, tb, n_fine, bcl, textlen=1e-3):
    """t and textbegin after n_fine steps of the reference driver loop (CellModel.h:405-420)."""
    for _ in range(n_fine):
        if t >= tb and t >= tb + textlen:
            tb += bcl
        t += DT
    return t, tb


def surrogate_leg(cm, torch, stream, steps, warmup, gen_frac=1.0):
    """Learned form: a surrogate trained here on the plain integrator's trajectories (untimed),
    then 1,048,576 jittered (+-15%) ten Tusscher cells paced at BCL 500 ms, timed over `steps`
    macro steps of 10 x 0.01 ms (one macro step = 10 cell-steps per cell)."""
    from cardiomechanics_gb300 import workloads as W
    t_train = time.perf_counter()
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    sur = cm.Surrogate(p, substeps=SUR_SUBSTEPS, seed=1, stream=stream.cuda_stream)
    pairs = 0
    for seed, bcl, beats in ((11, 0.5, 4), (12, 0.8, 3), (13, 1.0, 2)):  # three pacing rates
        tb_ = cm.Batch(p, 2048, cm.MIXED, stream=stream.cuda_stream)
        sc = W.conductance_scales(seed, 2048, 3, 0.85, 1.15)
        for k, name in enumerate(W.TT2_HETERO):
            tb_.add_hetero_value(name, p.get(name) * sc[k])
        v = tb_.init_vm()
        n_macro = int(round(beats * bcl / (SUR_SUBSTEPS * DT)) * gen_frac)
        pairs = sur.generate(tb_, v, n_macro, textlen=1e-3, bcl=bcl, amplitude=W.TT2_STIM_NA, cell_stride=4,
                             max_pairs=20_000_000)
    sur.fit(batch=4096, steps=max(1, int(6000 * gen_frac)), lr=1e-3, seed=1)
    loss = sur.fit(batch=8192, steps=max(1, int(4000 * gen_frac)), lr=3e-4, seed=2)
    t_train = time.perf_counter() - t_train
    b = cm.Batch(p, SUR_CELLS, cm.MIXED, stream=stream.cuda_stream)
    sc = W.conductance_scales(5, SUR_CELLS, 3, 0.85, 1.15)
    for k, name in enumerate(W.TT2_HETERO):
        b.add_hetero_value(name, p.get(name) * sc[k])
    vm = torch.tensor(b.init_vm(), device="cuda")
    kw = dict(textlen=1e-3, bcl=SUR_BCL, amplitude=W.TT2_STIM_NA, audit_mod=100)
    b.run_surrogate(sur, vm, warmup, t0=0.0, textbegin=0.0, **kw)
    t, tb = advance_protocol(0.0, 0.0, warmup * SUR_SUBSTEPS, SUR_BCL)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = b.run_surrogate(sur, vm, steps, t0=t, textbegin=tb, **kw)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    return {"value": SUR_CELLS * SUR_SUBSTEPS * steps / sec, "unit": UNIT, "cells": SUR_CELLS,
            "macro_steps": steps, "substeps": SUR_SUBSTEPS, "ms_per_macro_step": 1e3 * sec / steps,
            "bcl_ms": SUR_BCL * 1e3, "conductance_jitter": "g_Na,g_Kr,g_K1 x U[0.85,1.15]",
            "training": {"pairs": pairs, "final_normalised_mse": loss, "seconds": t_train},
            "stats": stats, "gpu_launches": 2 * steps}


BATCHED_SEED = 21
BATCHED_BCL = 1.0
# Algorithmic bytes per cell-step of the batched kernel (no per-cell conductances: each
# instance has its own parameter set): state planes and the Vm hi/lo pair read and written.
BATCHED_BYTES = {"TenTusscher2": 2 * 21 * 4 + 2 * 8, "CourtemancheEtAl": 2 * 25 * 4 + 2 * 8}


def batched_leg(cm, torch, stream, steps, warmup, hbm_peak, peak_kind):
    """Batched form: 256 instances (log-uniform 1k..1M cells, ten Tusscher 2006 or Courtemanche
    1998, own parameter set with six conductances x U[0.8, 1.2], stimulus phase U[0, BCL)),
    advanced in lock step by one persistent launch per step, replayed from a CUDA graph, launch
    shape autotuned on the instances. One step = one dt update of every cell of every instance."""
    from cardiomechanics_gb300 import workloads as W
    inst = W.batched_instances(BATCHED_SEED)
    batches, stims, vms = [], [], []
    for d in inst:
        p = cm.Params(d["model"], None, DT)
        for nm, sc in d["scales"].items():
            p.set(nm, p.get(nm) * sc)
        b = cm.Batch(p, d["n"], cm.MIXED, stream=stream.cuda_stream)
        batches.append(b)
        vms.append(torch.tensor(b.init_vm(), device="cuda"))
        tt2 = d["model"] == "TenTusscher2"
        stims.append({"textbegin": d["phase"] * BATCHED_BCL, "textlen": 1e-3 if tt2 else 2e-3, "bcl": BATCHED_BCL,
                      "amplitude": W.TT2_STIM_NA if tt2 else W.CRN_STIM_PAPF})
    multi = cm.Multi(batches, stream=stream.cuda_stream)
    tuned = multi.autotune(5)
    multi.run(vms, warmup, [dict(s, t0=0.0) for s in stims])
    timed = []
    for s in stims:
        t, tb = advance_protocol(0.0, s["textbegin"], warmup, s["bcl"], s["textlen"])
        timed.append(dict(s, t0=t, textbegin=tb))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    multi.run(vms, steps, timed)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    cells = sum(d["n"] for d in inst)
    algo = sum(d["n"] * BATCHED_BYTES[d["model"]] for d in inst)
    achieved = algo * steps / sec / 1e9
    out = {"value": cells * steps / sec, "unit": UNIT, "instances": len(inst), "cells": cells,
           "tt2_instances": sum(d["model"] == "TenTusscher2" for d in inst), "steps": steps,
           "ms_per_step": 1e3 * sec / steps, "bcl_ms": BATCHED_BCL * 1e3, "autotune": tuned,
           "sizes": "log-uniform [1e3, 1e6] seed %d" % BATCHED_SEED,
           "roofline": {"bound": "hbm", "kernel": "multi_kernel", "achieved": achieved, "peak": hbm_peak,
                        "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                        "algorithmic_bytes_per_step": algo},
           "gpu_launches": steps + 2 * len(inst)}
    del multi, batches
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=40)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", default="all", choices=["all", "mixed", "fp64", "e2e", "surrogate", "batched"],
                    help="run one leg only (for profiler captures); the JSON line is printed for 'all'")
    ap.add_argument("--tune-steps", type=int, default=10)
    ap.add_argument("--sur-steps", type=int, default=5000, help="timed macro steps of the learned form")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-steps", type=int, default=640, help="timed steps of the batched form")
    ap.add_argument("--sur-train-frac", type=float, default=1.0,
                    help="fraction of the surrogate's training run (profiling captures only; accuracy needs 1)")
    ap.add_argument("--launch", default=None, help="fixed mixed-kernel launch shape 'variant,grid_mode' (skips tuning)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import cardiomechanics_gb300 as cm

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    hbm_peak, peak_kind = peaks()

    if args.only == "surrogate":
        print(json.dumps(surrogate_leg(cm, torch, stream, args.sur_steps, 20, args.sur_train_frac)), flush=True)
        return
    if args.only == "batched":
        print(json.dumps(batched_leg(cm, torch, stream, args.batched_steps, 32, hbm_peak, peak_kind)), flush=True)
        return
    if args.only == "fp64":
        _, b64 = make_batch(cm, cm.FP64, stream.cuda_stream)
        vm64 = torch.tensor(b64.init_vm(), device="cuda")
        time_device_steps(torch, cm, b64, stream, vm64, args.fp64_steps, 3, 0.0)
        return
    # ---- device-resident mixed form (the headline `value`)
    p, b = make_batch(cm, cm.MIXED, stream.cuda_stream)
    if args.launch:
        v, g = (int(x) for x in args.launch.split(","))
        b.set_launch(v, g)
        tuned, tuned_ms = v * 100 + g, None
    else:
        tuned, tuned_ms = b.autotune(args.tune_steps)
    vm = torch.tensor(b.init_vm(), device="cuda")
    b.run(vm, args.warmup, textbegin=0.0, textlen=1e-3, bcl=BCL, amplitude=cm_stim())
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        b.run(vm, args.steps, t0=args.warmup * DT, textbegin=0.0, textlen=1e-3, bcl=BCL, amplitude=cm_stim())
        ev1.record(stream)
        torch.cuda.synchronize()
    sec = ev0.elapsed_time(ev1) / 1e3
    if world > 1:
        t = torch.tensor([sec], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        sec = float(t.item())
    value = world * N_CELLS * args.steps / sec
    audit = b.audit()
    ms_kernel = 1e3 * sec / args.steps
    if args.only == "mixed":
        return
    achieved = MIXED_BYTES_PER_CELL_STEP * N_CELLS / (ms_kernel / 1e3) / 1e9
    kernel = MIXED_KERNELS[tuned // 100] if 0 <= tuned // 100 < len(MIXED_KERNELS) else f"shape {tuned}"
    del b
    torch.cuda.empty_cache()

    fp64_peak = cm.fma_peak_tflops(True, stream.cuda_stream)
    fp32_peak = cm.fma_peak_tflops(False, stream.cuda_stream)
    # ---- plain FP64 kernel on the same workload
    _, b64 = make_batch(cm, cm.FP64, stream.cuda_stream)
    vm64 = torch.tensor(b64.init_vm(), device="cuda")
    sec64 = time_device_steps(torch, cm, b64, stream, vm64, args.fp64_steps, 3, 0.0)
    fp64_value = N_CELLS * args.fp64_steps / sec64
    fp64_ms = 1e3 * sec64 / args.fp64_steps
    del b64
    torch.cuda.empty_cache()

    # ---- end to end through the C ABI with pinned host buffers
    _, be = make_batch(cm, cm.MIXED, stream.cuda_stream)
    vm_h = torch.from_numpy(be.init_vm()).pin_memory()
    ie_h = torch.zeros(N_CELLS, dtype=torch.float64).pin_memory()
    amp = cm_stim()
    for s in range(3):
        ie_h.fill_(amp if s * DT <= 1e-3 else 0.0)
        be.calc_update(DT, vm_h, ie_h, None, vm_range=0.2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(args.e2e_steps):
        ie_h.fill_(amp if (s + 3) * DT <= 1e-3 else 0.0)
        be.calc_update(DT, vm_h, ie_h, None, vm_range=0.2)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    e2e_sec = max(wall, e0.elapsed_time(e1) / 1e3)
    e2e_value = N_CELLS * args.e2e_steps / e2e_sec
    del be

    sur = None
    if not args.no_surrogate:
        torch.cuda.empty_cache()
        sur = surrogate_leg(cm, torch, stream, args.sur_steps, 20)

    bat = None
    if not args.no_batched:
        torch.cuda.empty_cache()
        bat = batched_leg(cm, torch, stream, args.batched_steps, 32, hbm_peak, peak_kind)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(seconds=args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_kernel, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64acc", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": N_CELLS, "model": "TenTusscher2 epi", "dt_ms": DT * 1e3,
                       "bcl_ms": BCL * 1e3, "conductance_jitter": "g_Na,g_Kr,g_K1 x U[0.9,1.1] seed 2",
                       "precision": "mixed (FP32 gates/currents, compensated FP32 pairs for Vm/Na_i/K_i/CaSR)",
                       "l2": "state 430 MB > 129 MB L2 (no flush needed)", "parallelism": f"replicas{world}"},
            "plain_fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": fp64_ms, "steps": args.fp64_steps,
                           "bytes_per_cell_step": FP64_BYTES_PER_CELL_STEP,
                           "achieved_gbs": FP64_BYTES_PER_CELL_STEP * N_CELLS / (fp64_ms / 1e3) / 1e9,
                           "bound": "fp64 pipe", "fp64_fma_peak_tflops_measured": fp64_peak},
            "fp32_fma_peak_tflops_measured": fp32_peak,
            "autotune": {"choice": tuned, "ms_per_step": tuned_ms},
            "speedup_vs_plain_fp64": value / fp64_value,
            "surrogate_fp32": sur,
            "surrogate_speedup_vs_plain_fp64": (sur["value"] / fp64_value) if sur else None,
            "batched": bat,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 16 * N_CELLS,
                    "d2h_bytes_per_step": 8 * N_CELLS, "steps": args.e2e_steps,
                    "api": "cm_batch_step_update, pinned host Vm and i_ext"},
            "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                         "bytes_per_cell_step": MIXED_BYTES_PER_CELL_STEP,
                         "algorithmic_bytes_per_launch": MIXED_BYTES_PER_CELL_STEP * N_CELLS,
                         "traffic": MEASURED_TRAFFIC.get(kernel)},
            "cpu_baseline": cpu,
            "gpu_launches": args.steps + 2,  # the steps plus the Vm split/join of cm_batch_run
            "clocks": clk.summary(),
            "audit_mask": audit,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cm_stim():
    from cardiomechanics_gb300 import workloads as W
    return W.TT2_STIM_NA


if __name__ == "__main__":
    main()
