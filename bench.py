"""Benchmark of the cell-model update on GB300 (one JSON line on stdout).

Headline (`value`, `e2e`): the full chosen form at scale -- 16,777,216 ten Tusscher 2006
epicardial cells in 64 instances of uneven (log-uniform) size, each instance with its own
stimulus phase U[0, BCL) at BCL 500 ms (-52 pA/pF for 1 ms), g_Na/g_Kr/g_K1 jittered +-15 % per
cell, advanced by the learned macro step: 10 x 0.01 ms as one coarse physics step plus a
tensor-core MLP correction (FP32 state with compensated accumulators), the plain mixed
integrator for stimulated, fast (|dVm/dt| > 5 mV/ms) or rejected cells, and a rotating 1 %
audit sample integrated in FP64 on the device. One step = one macro step of every cell = 10
cell-steps per cell. The cells are packed into one batch (the instances share the parameter
set; per-cell stimulus times carry the phases). Inputs are synthetic (seeded); the state
(~2 GB) is larger than L2, so no flush is needed between steps.

value         cell-steps/s of the headline, state resident in HBM (CUDA events, batch stream)
e2e           the same through the C ABI with Vm in pinned HOST memory, one
              cm_batch_run_surrogate call per macro step (Vm read from and written to page-locked
              host memory by the macro-step kernels every step)
plain_fp64    the plain FP64 kernel (the reference's arithmetic) on the same 16.7M cells
roofline      the macro-step kernel (timed by the library's CUDA events) against measured HBM,
              with its tensor-core fraction beside it
precision_form  4,194,304 cells (2048 x 2048), FP32 + compensated accumulators, BCL 800 ms,
              +-10 %: the HBM-bound plain kernel with its own roofline
learned_form  1,048,576 cells, BCL 500 ms, +-15 %: the surrogate alone (mixed-precision audit)
batched       256 instances (1k-1M cells, TT2 and Courtemanche, own parameter sets and phases)
plain_small   65,536 cells in plain FP64 (the CPU-runnable case of the plain method)
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
# Launch shapes of cm_batch_set_launch (variant index -> kernel); 5 and 6 are bulk-copy staged,
# 7 and 8 the same with a producer warp and mbarrier hand-over.
MIXED_KERNELS = ["tt2_mixed_kernel<256>", "tt2_mixed_kernel<128>", "tt2_mixed_kernel<256,3>",
                 "tt2_mixed_kernel<512>", "tt2_mixed_kernel<64>", "mixed_staged_kernel<5,256>",
                 "mixed_staged_kernel<5,128>", "mixed_pipe_kernel<5,256,2>", "mixed_pipe_kernel<5,128,3>"]
# dram__bytes_read.sum + dram__bytes_write.sum of one launch on this workload, from ncu captures
# (launch shape 6, grid mode 4 and launch shape 7, grid mode 4).
MEASURED_TRAFFIC = {"mixed_staged_kernel<5,128>": 436_239_360 + 327_127_808,
                    "mixed_pipe_kernel<5,256,2>": 436_254_208 + 325_440_768}
# tt2_fp64_kernel: 18 FP64 states r+w (288 B), Vm r+w (16 B), 3 FP64 conductances (24 B).
FP64_BYTES_PER_CELL_STEP = 2 * 18 * 8 + 2 * 8 + 3 * 8
WORKLOAD = "tt2006-epi-precision-form-2048x2048"
# O'Hara-Rudy leg: 4,194,304 endocardial cells, INaF/IKr/IK1 multipliers x U[0.9, 1.1], -50 uA/uF
# x 1 ms every 1000 ms. Mixed form: 35 FP32 planes + 6 compensated pairs r+w (376 B), Vm pair r+w
# (16 B), 3 FP32 multipliers (12 B). FP64 form: 41 FP64 states r+w (656 B), Vm r+w (16 B), 3
# FP64 multipliers (24 B).
ORD_CELLS = 2048 * 2048
ORD_BCL = 1.0
ORD_MIXED_BYTES_PER_CELL_STEP = 2 * (35 + 12) * 4 + 2 * 2 * 4 + 3 * 4
ORD_FP64_BYTES_PER_CELL_STEP = 2 * 41 * 8 + 2 * 8 + 3 * 8
# Tomek: 38 FP32 states + 6 compensated pairs; 44 FP64 states (Vm pair and 3 multipliers as ORd)
TOM_MIXED_BYTES_PER_CELL_STEP = 2 * (38 + 12) * 4 + 2 * 2 * 4 + 3 * 4
TOM_FP64_BYTES_PER_CELL_STEP = 2 * 44 * 8 + 2 * 8 + 3 * 8
# The closed-form ventricular models timed beside the headline: the model's C-ABI id, the
# oracle's, its workload name, stimulus and bytes per cell step (mixed, FP64).
IONIC_LEGS = {
    "ohara_rudy": dict(model=12, oracle="ORD", label="ord2011", title="O'Hara-Rudy", stim="ORD_STIM",
                       het="ORD_HETERO", mixed_bytes=ORD_MIXED_BYTES_PER_CELL_STEP,
                       fp64_bytes=ORD_FP64_BYTES_PER_CELL_STEP),
    "tomek": dict(model=14, oracle="TOM", label="tomek2019", title="Tomek", stim="TOM_STIM", het="TOM_HETERO",
                  mixed_bytes=TOM_MIXED_BYTES_PER_CELL_STEP, fp64_bytes=TOM_FP64_BYTES_PER_CELL_STEP),
}
# Tissue leg (monodomain coupling): a 256 x 256 x 64 slab of TT2 epi cells on a 0.1 mm grid
# (D = 0.1 mm^2/ms, 7-point operator, no-flux faces), the x < 3 planes stimulated once. Mixed
# form per node-step: 21 state planes r+w (168 B), Vm hi/lo read + new hi/lo written (16 B), 3
# FP32 conductances (12 B), operator row: 7 entries x (4 B column + 4 B value) (56 B) + row sum
# (4 B), per-cell first-stimulus time (8 B), activation time read (8 B; written once per cell),
# neighbours' Vm from cache (counted once, 4 B).
TISSUE_DIMS = (256, 256, 64)
TISSUE_MIXED_BYTES = 168 + 16 + 12 + 56 + 4 + 8 + 8 + 4
# FP64 form: 18 states r+w (288 B), Vm r + w (16 B), 3 conductances (24 B), 7 x (4 + 8 B) (84 B),
# stimulus time (8 B), activation time (8 B), neighbours (8 B).
TISSUE_FP64_BYTES = 288 + 16 + 24 + 84 + 8 + 8 + 8
# The tissue leg with another cell model (--tissue-model): the same operator, stimulus protocol
# and per-node bytes with the model's own state planes (mixed: FP32 planes + pairs r+w; FP64:
# states r+w) in place of TT2's 168 / 288 B. Stimulus twice the model's single-cell amplitude.
TISSUE_MODELS = {
    "tt2": dict(model=5, label="tt2006-epi", het="TT2_HETERO", stim="TT2_STIM_NA", stim_text="2 x -52 pA/pF",
                mixed=TISSUE_MIXED_BYTES, fp64=TISSUE_FP64_BYTES),
    "ord": dict(model=12, label="ord2011-endo", het="ORD_HETERO", stim="ORD_STIM", stim_text="2 x -50 uA/uF",
                mixed=TISSUE_MIXED_BYTES - 168 + 2 * 47 * 4, fp64=TISSUE_FP64_BYTES - 288 + 2 * 41 * 8),
    "tomek": dict(model=14, label="tomek2019-endo", het="TOM_HETERO", stim="TOM_STIM", stim_text="2 x -53 uA/uF",
                  mixed=TISSUE_MIXED_BYTES - 168 + 2 * 50 * 4, fp64=TISSUE_FP64_BYTES - 288 + 2 * 44 * 8),
}
SUR_CELLS = 1 << 20   # the learned form (config 4)
SUR_BCL = 0.5
SUR_SUBSTEPS = 10     # fine steps per macro step
FULL_CELLS = 1 << 24
FULL_INSTANCES = 64
FULL_BCL = 0.5
FULL_SEED = 31       # instance sizes and phases
FULL_HET_SEED = 7    # per-cell conductances
FULL_AUDIT_MOD = 100
# Accuracy of the headline's own network: ACC_CELLS cells drawn from the headline population
# (seed ACC_SEED) run by the learned step and by the oracle over ACC_T_END seconds (five beats
# after every first stimulus), compared every macro step
ACC_SEED = 53
ACC_CELLS = 256
ACC_T_END = 3.0
ACC_BEATS = 5
FULL_WORKLOAD = "tt2006-epi-full-form-16.7M-cells-64-instances"
# Algorithmic bytes of one macro step: every cell's 21 state planes and Vm pair read and
# written plus 3 conductances read by sur_step (196 B), and the listed cells' 10 plain fine
# steps (196 B each) plus their list entry (4 B).
SUR_BYTES_PER_CELL = 2 * (21 * 4 + 2 * 4) + 3 * 4
SUR_PLAIN_BYTES_PER_LISTED_CELL = 10 * SUR_BYTES_PER_CELL + 4
# MLP FLOPs per cell of one macro step on the tensor core (padded shapes 32-128-128-32)
SUR_MLP_FLOPS_PER_CELL = 2 * (128 * 32 + 128 * 128 + 32 * 128)
# ncu: dram__bytes_read + dram__bytes_write of one macro-step launch over 4,194,304 cells (state
# 0.8 GB, six times the L2) on a plateau step, per cell: 0.94 of the algorithmic 196 B (the last
# tiles' writes are still in L2 when the launch ends); scaled by cells
SUR_STEP_TRAFFIC_PER_CELL = (441_412_864 + 330_322_944) / 4_194_304


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(torch, seconds, world, device="cuda"):
    """The replicas' timed region ends when the slowest rank's does: the maximum over ranks."""
    if world <= 1:
        return seconds
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


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


def bf16_peak():
    """(TFLOP/s, kind): the measured dense BF16 rate for a kernel timed inside a long step."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), "measured sustained"
    return 1700.0, "fallback sustained"


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


def headline_sample(k, seed=None):
    """k distinct cells of the headline population (seeded draw over the 16,777,216), with their
    conductance scales (3, k) and first stimulus times (their instance's phase x BCL)."""
    from cardiomechanics_gb300 import workloads as W
    seed = ACC_SEED if seed is None else seed
    draw = (W.uniform(seed, np.arange(4 * k, dtype=np.uint64)) * FULL_CELLS).astype(np.int64)
    _, first = np.unique(draw, return_index=True)
    idx = draw[np.sort(first)[:k]]  # the first k distinct cells in draw order
    inst = W.full_form_instances(FULL_SEED, FULL_INSTANCES, FULL_CELLS)
    ends = np.cumsum([d["n"] for d in inst])
    phases = np.array([inst[i]["phase"] for i in np.searchsorted(ends, idx, side="right")]) * FULL_BCL
    sc = W.conductance_scales(FULL_HET_SEED, FULL_CELLS, 3, 0.85, 1.15, cells=idx)
    return idx, sc, phases


def cpu_model():
    """The host CPU's model name (lscpu), for the baseline's description."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


class CPUSample:
    """The oracle (C restatement of the reference Calc, FP64: the reference's plain method) on a
    bounded sample of the headline workload: `cells` cells drawn from its 16,777,216 (seeded),
    each with its own conductances and its instance's first stimulus time, all host threads."""

    def __init__(self, cells=4096, threads=None):
        import oracle as O
        from cardiomechanics_gb300 import workloads as W
        self.O, self.W = O, W
        self.port = O.Port()
        self.threads = threads or os.cpu_count() or 1
        self.cells = cells
        self.P = self.port.param_vector(O.TT2, O.load_params(O.TT2))
        self.T = self.port.tables(O.TT2, self.P, DT)
        _, sc, self.tb = headline_sample(cells)
        names = self.port.param_names(O.TT2)
        self.het = {k: self.P[names.index(k)] * sc[i] for i, k in enumerate(W.TT2_HETERO)}
        self.B = self.port.init_state(O.TT2, self.P, cells)
        self.vm = np.full(cells, self.port.init_vm(O.TT2, self.P))
        self.t = 0.0

    def advance(self, steps, rows=None, rec_every=0):
        """Advance the sample (or its rows `rows`) `steps` steps of the driver loop; returns
        (elapsed seconds, Vm trace of the rows when rec_every > 0)."""
        sl = slice(None) if rows is None else rows
        B = np.ascontiguousarray(self.B[sl])
        vm = np.ascontiguousarray(self.vm[sl])
        tb = np.ascontiguousarray(self.tb[sl])
        het = {k: np.ascontiguousarray(v[sl]) for k, v in self.het.items()}
        t0 = time.perf_counter()
        tr = self.port.run(self.O.TT2, self.P, self.T, B, vm, steps, DT, t0=self.t, textlen=1e-3, bcl=FULL_BCL,
                           amp=self.W.TT2_STIM_NA, het=het, textbegin_per_cell=tb, rec_every=rec_every,
                           n_threads=self.threads)
        el = time.perf_counter() - t0
        self.B[sl], self.vm[sl] = B, vm
        if rows is None:  # the driver's protocol state after these steps (the port only reads it)
            t = self.t
            for _ in range(steps):
                adv = (t >= self.tb) & (t >= self.tb + 1e-3)
                self.tb = np.where(adv, self.tb + FULL_BCL, self.tb)
                t += DT
            self.t = t
        return el, tr

    def describe(self, cell_steps, seconds, what):
        return {"unit": UNIT, "cores": self.threads, "kind": "port", "cpu": cpu_model(),
                "sample": f"{self.cells} of the {FULL_CELLS} headline cells (seeded draw, own conductances and "
                          f"stimulus phases), {what}: {cell_steps:.3g} cell-steps of the oracle C restatement of "
                          f"the reference Calc in FP64 on {self.threads} threads, {seconds:.1f} s"}


def cpu_baseline(cells=4096):
    """Oracle throughput on the host cores over the accuracy protocol (3.0 s simulated: five
    beats after every first stimulus) for `cells` headline cells; the first ACC_CELLS of them
    are recorded every macro step and returned as the FP64 reference of the accuracy check."""
    smp = CPUSample(cells)
    steps = int(round(ACC_T_END / DT))
    el_a, traces = smp.advance(steps, rows=slice(0, ACC_CELLS), rec_every=SUR_SUBSTEPS)
    el_b, _ = smp.advance(steps, rows=slice(ACC_CELLS, cells))
    el = el_a + el_b
    d = smp.describe(cells * steps, el, f"{ACC_T_END:.1f} s simulated")
    d["value"] = cells * steps / el
    return d, traces


def run_reference(args):
    """The reference arm: the reference's CPU path (the oracle port of its Calc; the reference
    sources are not on the GPU host) on all host cores, on the headline's config. One step
    advances a sample of the headline cells by a chunk of fine steps sized so that warmup +
    steps take about a minute and a half; ms_per_step is that step's own measured time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle as O
    O.build_port()
    smp = CPUSample(4096)
    el, _ = smp.advance(200)  # calibration
    rate = smp.cells * 200 / el
    total = args.steps + args.warmup
    chunk = int(max(1, min(5000, rate * 90.0 / max(1, total) / smp.cells)))
    for _ in range(args.warmup):
        smp.advance(chunk)
    times = [smp.advance(chunk)[0] for _ in range(args.steps)]
    v = float(np.median([smp.cells * chunk / t for t in times]))
    cb = smp.describe(smp.cells * chunk * args.steps, float(sum(times)), f"{chunk} fine steps per timed step")
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.median(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(world),
            "method": "the reference's plain FP64 Rush-Larsen Calc (oracle restatement), all host cores",
            "step": f"one step advances {smp.cells} headline cells by {chunk} fine steps of 0.01 ms",
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def headline_config(world):
    """The headline's `config` (the same dict on both arms)."""
    from cardiomechanics_gb300 import workloads as W
    sizes = np.array([d["n"] for d in W.full_form_instances(FULL_SEED, FULL_INSTANCES, FULL_CELLS)])
    return {"workload": FULL_WORKLOAD, "cells": FULL_CELLS,
            "instances": {"n": FULL_INSTANCES, "min_cells": int(sizes.min()), "max_cells": int(sizes.max())},
            "model": "TenTusscher2 epi", "dt_ms": DT * 1e3, "macro_step_ms": SUR_SUBSTEPS * DT * 1e3,
            "cell_steps_per_step": FULL_CELLS * SUR_SUBSTEPS, "bcl_ms": FULL_BCL * 1e3,
            "stimulus": "-52 pA/pF x 1 ms, per-instance phase U[0, BCL)",
            "conductance_jitter": "g_Na,g_Kr,g_K1 x U[0.85,1.15] per cell",
            "method": "learned macro step (coarse step + 22-128-128-19 BF16 MLP on tcgen05), "
                      "plain FP32 fallback, 1% FP64 audit",
            "l2": "state ~2 GB > 129 MB L2 (no flush needed)", "parallelism": f"replicas{world}"}


def advance_protocol(t, tb, n_fine, bcl, textlen=1e-3):
    """t and textbegin after n_fine steps of the reference driver loop (CellModel.h:405-420)."""
    for _ in range(n_fine):
        if t >= tb and t >= tb + textlen:
            tb += bcl
        t += DT
    return t, tb


def train_surrogate(cm, stream, seeds=(1, 2, 3)):
    """The surrogate used by the learned legs, trained here (untimed) on the plain integrator's
    trajectories and selected on held-out cells (`learned.train_and_select`: one dataset,
    one network per seed, three correction sets each, the candidate with the smallest trace error
    against the FP64 kernel kept). Deterministic: the same seeds give the same network."""
    from cardiomechanics_gb300 import learned as L
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    sur = cm.Surrogate(p, substeps=SUR_SUBSTEPS, seed=1, stream=stream.cuda_stream)
    if not seeds:  # profiler captures only: an untrained network with a zero output layer
        prm = sur.mlp.get_params()
        prm[4][:] = 0.0
        prm[5][:] = 0.0
        sur.mlp.set_params(prm)
        return p, sur, {"untrained": "zero output layer (capture run: the step equals the coarse step)"}
    rep = L.train_and_select(cm, p, sur, seeds=seeds, stream=stream)
    applied = sur.get_blob()[L.APPLIED]
    rep["corrected_outputs"] = [nm for nm, a in zip(L.OUTPUT_NAMES, applied) if a > 0]
    return p, sur, rep


def learned_leg(cm, torch, stream, p, sur, steps, warmup, cells=None):
    """Learned form: 1,048,576 jittered (+-15 %) ten Tusscher cells paced together at BCL 500 ms,
    timed over `steps` macro steps of 10 x 0.01 ms (one macro step = 10 cell-steps per cell),
    mixed-precision audit of 1 % of the cells."""
    from cardiomechanics_gb300 import workloads as W
    n_cells = cells or SUR_CELLS
    b = cm.Batch(p, n_cells, cm.MIXED, stream=stream.cuda_stream)
    sc = W.conductance_scales(5, n_cells, 3, 0.85, 1.15)
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
    return {"value": n_cells * SUR_SUBSTEPS * steps / sec, "unit": UNIT, "cells": n_cells,
            "macro_steps": steps, "substeps": SUR_SUBSTEPS, "ms_per_macro_step": 1e3 * sec / steps,
            "bcl_ms": SUR_BCL * 1e3, "conductance_jitter": "g_Na,g_Kr,g_K1 x U[0.85,1.15]",
            "audit": "1 % rotating, mixed precision", "stats": stats, "gpu_launches": 2 * steps + 2}


def full_form_population(cm, p, precision, stream):
    """The headline population: one batch of FULL_CELLS cells (64 instances packed), per-cell
    conductances, per-cell first stimulus times (the instance's phase)."""
    from cardiomechanics_gb300 import workloads as W
    inst = W.full_form_instances(FULL_SEED, FULL_INSTANCES, FULL_CELLS)
    b = cm.Batch(p, FULL_CELLS, precision, stream=stream.cuda_stream)
    sc = W.conductance_scales(FULL_HET_SEED, FULL_CELLS, 3, 0.85, 1.15)
    for k, name in enumerate(W.TT2_HETERO):
        b.add_hetero_value(name, p.get(name) * sc[k])
    del sc
    return inst, b


def full_form_leg(cm, torch, stream, p, sur, steps, warmup, e2e_steps, fp64_steps, hbm_peak, peak_kind,
                  barrier=lambda: None):
    """The headline: see the module docstring. Returns the leg's figures."""
    from cardiomechanics_gb300 import workloads as W
    inst, b = full_form_population(cm, p, cm.MIXED, stream)
    sizes = np.array([d["n"] for d in inst])
    for d in inst:
        d["tb"] = d["phase"] * FULL_BCL
    kw = dict(textlen=1e-3, bcl=FULL_BCL, amplitude=W.TT2_STIM_NA, mode=cm.SUR_AUDIT_FP64, audit_mod=FULL_AUDIT_MOD)

    def tb_cells(tbs):
        return torch.tensor(np.repeat(np.array(tbs), sizes), dtype=torch.float64, device="cuda")

    vm = torch.tensor(b.init_vm(), device="cuda")
    # per-cell first stimulus times on the device: each run advances them in place (driver state)
    tbc = tb_cells([d["tb"] for d in inst])
    b.run_surrogate(sur, vm, warmup, t0=0.0, textbegin_per_cell=tbc, **kw)
    t = advance_protocol(0.0, 0.0, warmup * SUR_SUBSTEPS, 1e9)[0]
    torch.cuda.synchronize()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        stats = b.run_surrogate(sur, vm, steps, t0=t, textbegin_per_cell=tbc, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    t = advance_protocol(t, 0.0, steps * SUR_SUBSTEPS, 1e9)[0]
    # ---- the same window with the coarse step alone (the method without the network)
    c0 = torch.cuda.Event(enable_timing=True)
    c1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    c0.record(stream)
    stats_c = b.run_surrogate(sur, vm, steps, t0=t, textbegin_per_cell=tbc,
                              **dict(kw, mode=cm.SUR_COARSE_ONLY | cm.SUR_AUDIT_FP64))
    c1.record(stream)
    torch.cuda.synchronize()
    sec_c = c0.elapsed_time(c1) / 1e3
    t = advance_protocol(t, 0.0, steps * SUR_SUBSTEPS, 1e9)[0]
    value = FULL_CELLS * SUR_SUBSTEPS * steps / sec
    ms = 1e3 * sec / steps
    listed = stats["fallback"] / max(1, steps)  # cells the plain integrator advanced per macro step
    # the macro-step kernel alone, timed by the library's events around each of its launches
    ms_k = stats["ms_step_kernel"] / steps
    ms_p = stats["ms_plain_kernel"] / steps
    algo = FULL_CELLS * SUR_BYTES_PER_CELL
    achieved = algo / (ms_k / 1e3) / 1e9
    tflops = FULL_CELLS * SUR_MLP_FLOPS_PER_CELL / (ms_k / 1e3) / 1e12
    tpk, tpk_kind = bf16_peak()

    # ---- end to end: one C-ABI call per macro step with the cells' Vm in pinned HOST memory
    # (read and written there by the call's kernels); the stimulus times stay on the device
    vm_h = vm.cpu().pin_memory()
    del vm
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    e2e_fb = e2e_cms = 0
    for _ in range(e2e_steps):
        st = b.run_surrogate(sur, vm_h, 1, t0=t, textbegin_per_cell=tbc, **kw)
        e2e_fb += st["fallback"]
        e2e_cms += st["cell_macro_steps"]
        for _k in range(SUR_SUBSTEPS):
            t += DT
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_sec = max(time.perf_counter() - w0, f0.elapsed_time(f1) / 1e3)
    del b, tbc
    torch.cuda.empty_cache()

    # ---- plain FP64 kernel on the same cells and protocol
    _, b64 = full_form_population(cm, p, cm.FP64, stream)
    v64 = torch.tensor(b64.init_vm(), device="cuda")
    tb64 = tb_cells([d["phase"] * FULL_BCL for d in inst])
    b64.run(v64, 3, textlen=1e-3, bcl=FULL_BCL, amplitude=W.TT2_STIM_NA, textbegin_per_cell=tb64)
    torch.cuda.synchronize()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    b64.run(v64, fp64_steps, t0=3 * DT, textlen=1e-3, bcl=FULL_BCL, amplitude=W.TT2_STIM_NA, textbegin_per_cell=tb64)
    g1.record(stream)
    torch.cuda.synchronize()
    sec64 = g0.elapsed_time(g1) / 1e3
    del b64, v64
    torch.cuda.empty_cache()
    fp64_value = FULL_CELLS * fp64_steps / sec64

    # ---- accuracy of this network on ACC_CELLS cells of this population (own conductances and
    # phases), five beats, every macro step: learned step and coarse step alone; the FP64 kernel
    # on the same cells (the oracle's traces come from the CPU leg)
    from cardiomechanics_gb300 import learned as L
    idx, _, ph = headline_sample(ACC_CELLS)
    acc_tr, acc_stats = {}, {}
    for name, mode in (("learned", cm.SUR_AUDIT_FP64), ("coarse_only", cm.SUR_COARSE_ONLY | cm.SUR_AUDIT_FP64)):
        acc_tr[name], acc_stats[name] = L.surrogate_traces(cm, p, sur, ACC_CELLS, FULL_HET_SEED, ph, ACC_T_END, 1,
                                                           mode, stream, cells=idx, audit_mod=FULL_AUDIT_MOD)
    ref64 = L.fp64_traces(cm, p, ACC_CELLS, FULL_HET_SEED, ph, ACC_T_END, 1, stream, cells=idx)
    vs_kernel = {k: L.trace_errors(v, ref64, ph, SUR_SUBSTEPS * DT, ACC_BEATS) for k, v in acc_tr.items()}
    return {
        "value": value, "seconds": sec, "ms_per_step": ms, "stats": stats, "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "kernel": "sur_step_tc_kernel<4, audit> (4 groups; group 3 audits first)",
                     "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                     "ms_per_launch": ms_k, "algorithmic_bytes_per_launch": algo,
                     "traffic": SUR_STEP_TRAFFIC_PER_CELL * FULL_CELLS,
                     "traffic_note": "ncu DRAM read+write bytes of one 4,194,304-cell launch on a plateau step, "
                                     "scaled by cells: 0.94 of the algorithmic bytes",
                     "algorithmic_bytes_note": "196 B per cell: 21 state planes and the Vm pair read and written, "
                                               "3 conductances read; the 8 B per-cell first-stimulus time the step "
                                               "also reads is not counted",
                     "tensor": {"achieved": tflops, "peak": tpk, "unit": "TFLOP/s", "frac": tflops / tpk,
                                "peak_kind": tpk_kind, "flops_per_launch": FULL_CELLS * SUR_MLP_FLOPS_PER_CELL},
                     "bound_note": "issue-bound: neither HBM nor the tensor pipe limits this kernel"},
        "sur_plain_kernel": {"ms_per_launch": ms_p, "listed_cells_per_launch": listed,
                             "algorithmic_bytes_per_launch": listed * SUR_PLAIN_BYTES_PER_LISTED_CELL},
        "e2e": {"value": FULL_CELLS * SUR_SUBSTEPS * e2e_steps / e2e_sec, "unit": UNIT,
                "h2d_bytes_per_step": 8 * FULL_CELLS, "d2h_bytes_per_step": 8 * FULL_CELLS, "steps": e2e_steps,
                "fallback_fraction": e2e_fb / max(1, e2e_cms),
                "api": "cm_batch_run_surrogate per macro step, Vm in pinned host memory; per-cell stimulus "
                       "times kept on the device (advanced in place by the library)"},
        "plain_fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": 1e3 * sec64 / fp64_steps,
                       "steps": fp64_steps, "cells": FULL_CELLS, "bytes_per_cell_step": FP64_BYTES_PER_CELL_STEP,
                       "achieved_gbs": FP64_BYTES_PER_CELL_STEP * FULL_CELLS / (sec64 / fp64_steps) / 1e9,
                       "bound": "fp64 pipe"},
        "gpu_launches": 2 * steps + 2,
        "instances": {"n": FULL_INSTANCES, "min_cells": int(sizes.min()), "max_cells": int(sizes.max())},
        "fallback_fraction": stats["fallback"] / (FULL_CELLS * steps),
        "coarse_only": {"value": FULL_CELLS * SUR_SUBSTEPS * steps / sec_c, "unit": UNIT, "ms_per_step": 1e3 * sec_c / steps,
                        "fallback_fraction": stats_c["fallback"] / (FULL_CELLS * steps),
                        "note": "the same timed window and cells with the coarse step alone (no network)"},
        "accuracy_traces": acc_tr, "accuracy_stats": acc_stats, "accuracy_phases": ph,
        "accuracy_vs_fp64_kernel": vs_kernel,
    }


BATCHED_SEED = 21
BATCHED_BCL = 1.0
# Algorithmic bytes per cell-step of the batched kernel (no per-cell conductances: each
# instance has its own parameter set): state planes and the Vm hi/lo pair read and written.
MULTI_KERNELS = ["multi_kernel<256>", "multi_kernel<128>", "multi_kernel<512>", "multi_staged_kernel<128>",
                 "multi_staged_kernel<256>", "multi_pipe_kernel<256,2>", "multi_pipe_kernel<128,3>",
                 "multi_pipe_kernel<256,3>", "multi_pipe_kernel<128,4>"]
BATCHED_BYTES = {"TenTusscher2": 2 * 21 * 4 + 2 * 8, "CourtemancheEtAl": 2 * 25 * 4 + 2 * 8}


def batched_leg(cm, torch, stream, steps, warmup, hbm_peak, peak_kind, n_inst=256, launch=None):
    """Batched form: 256 instances (log-uniform 1k..1M cells, ten Tusscher 2006 or Courtemanche
    1998, own parameter set with six conductances x U[0.8, 1.2], stimulus phase U[0, BCL)),
    advanced in lock step by one persistent launch per step, replayed from a CUDA graph, launch
    shape autotuned on the instances. One step = one dt update of every cell of every instance."""
    from cardiomechanics_gb300 import workloads as W
    inst = W.batched_instances(BATCHED_SEED, n_inst)
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
    if launch:  # tile_cells,shape,blocks_per_sm (profiler captures)
        tc, sh, bps = (int(x) for x in launch.split(","))
        multi.set_launch(tc, sh, bps)
        tuned = {"tile_cells": tc, "shape": sh, "blocks_per_sm": bps, "ms_per_step": None}
    else:
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
           "roofline": {"bound": "hbm", "kernel": MULTI_KERNELS[tuned["shape"]] if 0 <= tuned["shape"] < len(MULTI_KERNELS)
                        else "multi shape %d" % tuned["shape"], "achieved": achieved, "peak": hbm_peak,
                        "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                        "algorithmic_bytes_per_step": algo},
           "gpu_launches": steps + 2 * len(inst)}
    del multi, batches
    return out


def plain_small_leg(cm, torch, stream, steps=2000):
    """The plain method's small case: 65,536 TT2 epi cells in FP64 (the reference arithmetic),
    g_Na/g_Kr/g_K1 x U[0.95, 1.05] (seed 1), -52 pA/pF for 1 ms every 1000 ms, timed over
    `steps` of the 100,000-step (1000 ms) run."""
    from cardiomechanics_gb300 import workloads as W
    n = 65536
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    b = cm.Batch(p, n, cm.FP64, stream=stream.cuda_stream)
    sc = W.conductance_scales(1, n, 3, 0.95, 1.05)
    for k, name in enumerate(W.TT2_HETERO):
        b.add_hetero_value(name, p.get(name) * sc[k])
    vm = torch.tensor(b.init_vm(), device="cuda")
    kw = dict(textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=W.TT2_STIM_NA)
    b.run(vm, 20, **kw)
    t = advance_protocol(0.0, 0.0, 20, 1e9)[0]
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.run(vm, steps, t0=t, **kw)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    return {"value": n * steps / sec, "unit": UNIT, "cells": n, "steps": steps, "ms_per_step": 1e3 * sec / steps,
            "precision": "FP64", "conductance_jitter": "g_Na,g_Kr,g_K1 x U[0.95,1.05] seed 1", "bcl_ms": 1000.0,
            "note": "65,536 cells leave most of the GPU's FP64 pipes idle; the 4.2M-cell figure is plain_fp64"}


CRN_CELLS = 2048 * 2048
# Courtemanche single-batch kernels: mixed 17 FP32 states + 4 compensated pairs r+w (200 B), Vm
# pair r+w (16 B), 3 FP32 conductances (12 B); FP64 21 states r+w (336 B), Vm r+w (16 B), 3 FP64
# conductances (24 B)
CRN_MIXED_BYTES_PER_CELL_STEP = 2 * (17 + 8) * 4 + 2 * 8 + 3 * 4
CRN_FP64_BYTES_PER_CELL_STEP = 2 * 21 * 8 + 2 * 8 + 3 * 8


def crn_leg(cm, torch, stream, args, hbm_peak, peak_kind):
    """Courtemanche 1998 single-batch kernels: 4,194,304 atrial cells, g_Na/g_to/g_CaL x U[0.9,
    1.1], 20 pA/pF for 2 ms every 1000 ms; the mixed form at each launch shape the autotuner
    tries on it (the autotuner's pick reported) and the FP64 form, each with its HBM fraction."""
    from cardiomechanics_gb300 import workloads as W
    n = args.crn_cells
    p = cm.Params(cm.COURTEMANCHE, None, DT)
    out = {"cells": n, "bcl_ms": 1000.0}
    for prec, steps, nbytes in ((cm.MIXED, args.crn_steps, CRN_MIXED_BYTES_PER_CELL_STEP),
                                (cm.FP64, max(3, args.crn_steps // 50), CRN_FP64_BYTES_PER_CELL_STEP)):
        b = cm.Batch(p, n, prec, stream=stream.cuda_stream)
        sc = W.conductance_scales(4, n, 3, 0.9, 1.1)
        for k, name in enumerate(W.CRN_HETERO):
            b.add_hetero_value(name, p.get(name) * sc[k])
        shape = None
        if prec == cm.MIXED:
            shape = b.autotune(args.tune_steps)[0] if args.launch is None else None
            if args.launch is not None:
                v, g = (int(x) for x in args.launch.split(","))
                b.set_launch(v, g)
                shape = v * 100 + g
        vm = torch.tensor(b.init_vm(), device="cuda")
        kw = dict(textbegin=0.0, textlen=2e-3, bcl=1.0, amplitude=W.CRN_STIM_PAPF)
        b.run(vm, 3, **kw)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(vm, steps, t0=3 * DT, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        gbs = nbytes * n * steps / sec / 1e9
        key = "mixed" if prec == cm.MIXED else "fp64"
        out[key] = {"value": n * steps / sec, "unit": UNIT, "steps": steps, "ms_per_step": 1e3 * sec / steps,
                    "bytes_per_cell_step": nbytes, "achieved_gbs": gbs, "hbm_frac": gbs / hbm_peak,
                    "peak_kind": peak_kind, "launch_shape": shape}
        del b, vm
        torch.cuda.empty_cache()
    return out


def training_leg(cm, torch, stream, args):
    """The surrogate's training kernels alone (profiler captures): the dataset generation
    (plain mixed steps, pair recording, ordered append) and one network's fit, each timed."""
    from cardiomechanics_gb300 import learned as L
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    sur = cm.Surrogate(p, substeps=SUR_SUBSTEPS, seed=1, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pairs = L.generate(cm, p, sur, stream, args.gen_steps)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    steps = args.fit_steps
    sur.reset_network(1)
    loss = sur.fit(batch=4096, steps=steps, lr=1e-3, seed=3)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"pairs": pairs, "generate_s": t1 - t0, "fit_steps": steps, "fit_s": t2 - t1,
            "ms_per_adam_step": 1e3 * (t2 - t1) / max(1, steps), "loss": loss, "batch": 4096}


class IonicCPUSample:
    """The oracle's restatement of a closed-form ventricular model (O'Hara-Rudy or Tomek, the
    reference Calc in FP64) on the first `cells` cells of that model's leg, all host threads."""

    def __init__(self, leg, cells=2048, threads=None):
        import oracle as O
        from cardiomechanics_gb300 import workloads as W
        self.O, self.W, self.port = O, W, O.Port()
        self.spec = IONIC_LEGS[leg]
        self.m = getattr(O, self.spec["oracle"])
        self.stim = getattr(W, self.spec["stim"])
        self.threads = threads or os.cpu_count() or 1
        self.cells = cells
        self.P = self.port.param_vector(self.m, O.load_params(self.m, "endo"))
        sc = W.conductance_scales(3, ORD_CELLS, 3, 0.9, 1.1, cells=np.arange(cells))
        names = self.port.param_names(self.m)
        self.het = {k: self.P[names.index(k)] * sc[i] for i, k in enumerate(getattr(W, self.spec["het"]))}
        self.B = self.port.init_state(self.m, self.P, cells)
        self.vm = np.full(cells, self.port.init_vm(self.m, self.P))

    def rate(self, seconds):
        done, el, t = 0, 0.0, 0.0
        while el < seconds:
            t0 = time.perf_counter()
            self.port.run(self.m, self.P, np.zeros((0, self.O.RTDT)), self.B, self.vm, 200, DT, t0=t,
                          textbegin=0.0, textlen=1e-3, bcl=1e9, amp=self.stim, het=self.het,
                          n_threads=self.threads)
            el += time.perf_counter() - t0
            done += 200
            t += 200 * DT
        return {"value": self.cells * done / el, "unit": UNIT, "cores": self.threads, "kind": "port",
                "sample": f"first {self.cells} of the {ORD_CELLS} {self.spec['title']} cells x {done} steps of "
                          f"0.01 ms (oracle C restatement of the reference Calc in FP64, {self.threads} threads, "
                          f"{el:.1f} s)"}


def ionic_leg(cm, torch, stream, args, hbm_peak, peak_kind, leg, fp64_peak=None, cpu_seconds=0.0):
    """A closed-form ventricular model (O'Hara-Rudy 2011 or Tomek 2019, the reference's
    variants), 4,194,304 endocardial cells: the mixed form (autotuned launch shape) and the
    plain FP64 form, each timed with events on its stream."""
    from cardiomechanics_gb300 import workloads as W
    spec = IONIC_LEGS[leg]
    stim = getattr(W, spec["stim"])
    hetn = getattr(W, spec["het"])
    n = args.ord_cells
    p = cm.Params(spec["model"], None, DT)
    sc = W.conductance_scales(3, n, 3, 0.9, 1.1)
    kw = dict(textbegin=0.0, textlen=1e-3, bcl=ORD_BCL, amplitude=stim)
    out = {"workload": f"{spec['label']}-endo-{n}-cells", "cells": n, "bcl_ms": ORD_BCL * 1e3,
           "conductance_jitter": "INaF,IKr,IK1 multipliers x U[0.9,1.1] seed 3",
           "stimulus": f"{stim:g} uA/uF x 1 ms"}
    for prec, steps, name in ((cm.MIXED, args.ord_steps, "mixed"), (cm.FP64, args.fp64_steps, "fp64")):
        b = cm.Batch(p, n, prec, stream=stream.cuda_stream)
        for k, h in enumerate(hetn):
            b.add_hetero_value(h, p.get(h) * sc[k])
        tuned = None
        if prec == cm.MIXED and args.launch:
            v, g = (int(x) for x in args.launch.split(","))
            b.set_launch(v, g)
            tuned = (f"{v},{g} (fixed)", None)
        elif prec == cm.MIXED:
            tuned = b.autotune(args.tune_steps)
        vm = torch.tensor(b.init_vm(), device="cuda")
        b.run(vm, 3, **kw)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(vm, steps, t0=3 * DT, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        bps = spec["mixed_bytes"] if prec == cm.MIXED else spec["fp64_bytes"]
        achieved = bps * n * steps / sec / 1e9
        res = {"value": n * steps / sec, "unit": UNIT, "steps": steps, "ms_per_step": 1e3 * sec / steps,
               "audit_mask": b.audit(), "gpu_launches": steps,
               "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                       "peak_kind": peak_kind, "bytes_per_cell_step": bps}}
        if tuned is not None:
            res["autotune"] = {"choice": tuned[0], "ms_per_step": tuned[1]}
            res["precision"] = "mixed (FP32 gates/currents, compensated FP32 pairs for Vm, Na_i, Na_ss, K_i, " \
                               "K_ss, Ca_nsr, Ca_jsr)"
        else:
            res["precision"] = "FP64 (the reference arithmetic)"
            if fp64_peak:
                res["fp64_fma_peak_tflops_measured"] = fp64_peak
        out[name] = res
        del b, vm
        torch.cuda.empty_cache()
    out["mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    if cpu_seconds > 0:
        out["cpu_baseline"] = IonicCPUSample(leg).rate(cpu_seconds)
    return out


def tissue_leg(cm, torch, stream, args, hbm_peak, peak_kind):
    """Monodomain coupling: the intra product fused with the TT2 update, Godunov step, range check
    and activation times (cm_batch_run_diffuse) on a 4,194,304-node slab; the same step split
    into cm_diffusion_apply + cm_batch_step_update_act beside it; the FP64 form."""
    from cardiomechanics_gb300 import workloads as W
    tm = TISSUE_MODELS[args.tissue_model]
    hetn = getattr(W, tm["het"])
    nx, ny, nz = TISSUE_DIMS if args.tissue_dims is None else tuple(args.tissue_dims)
    n = nx * ny * nz
    rp, col, val = W.grid_laplacian(nx, ny, nz)
    d = cm.Diffusion(rp, col, val, uniform_scale=W.COUPLING_SCALE[tm["model"]])
    del rp, col, val
    p = cm.Params(tm["model"], None, DT)
    sc = W.conductance_scales(5, n, 3, 0.95, 1.05)
    tb = torch.tensor(np.where(np.arange(n) % nx < 3, 0.0, 1e9), device="cuda")
    amp = 2 * getattr(W, tm["stim"])
    out = {"workload": f"{tm['label']}-slab-{nx}x{ny}x{nz}", "nodes": n, "grid_mm": 0.1, "D_mm2_per_ms": 0.1,
           "operator": "7-point finite differences, no-flux faces",
           "stimulus": f"x < 3 planes, {tm['stim_text']} x 1 ms"}
    kw = dict(textlen=1e-3, bcl=1e9, amplitude=amp, act_threshold=-0.02, vm_range=0.2)
    for prec, steps, name in ((cm.MIXED, args.tissue_steps, "fused_mixed"), (cm.FP64, args.fp64_steps, "fused_fp64")):
        b = cm.Batch(p, n, prec, stream=stream.cuda_stream)
        for k, h in enumerate(hetn):
            b.add_hetero_value(h, p.get(h) * sc[k])
        if prec == cm.MIXED and args.launch:  # 5 or 6: the double-buffered staged kernel
            b.set_launch(*(int(x) for x in args.launch.split(",")))
        vm = torch.tensor(b.init_vm(), device="cuda")
        act = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
        tbc = tb.clone()
        b.run_diffuse(d, vm, 3, textbegin_per_cell=tbc, act=act, **kw)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run_diffuse(d, vm, steps, t0=3 * DT, textbegin_per_cell=tbc, act=act, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        bps = tm["mixed"] if prec == cm.MIXED else tm["fp64"]
        achieved = bps * n * steps / sec / 1e9
        out[name] = {"value": n * steps / sec, "unit": UNIT, "steps": steps, "ms_per_step": 1e3 * sec / steps,
                     "activated": int((act >= 0).sum().item()), "audit_mask": b.audit(),
                     "gpu_launches": steps + 2,
                     "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                             "peak_kind": peak_kind, "bytes_per_node_step": bps}}
        del b, vm, act
        torch.cuda.empty_cache()
    # the split form a caller would write without the fused entry point (mixed batch, device arrays)
    b = cm.Batch(p, n, cm.MIXED, stream=stream.cuda_stream)
    for k, h in enumerate(hetn):
        b.add_hetero_value(h, p.get(h) * sc[k])
    vm = torch.tensor(b.init_vm(), device="cuda")
    act = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    iext = torch.zeros(n, dtype=torch.float64, device="cuda")
    steps = max(10, args.tissue_steps // 5)
    for k in range(3):
        d.apply(vm, iext)
        b.calc_update_act(DT, vm, act, k * DT, -0.02, i_ext=iext)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(steps):
        d.apply(vm, iext)
        b.calc_update_act(DT, vm, act, (3 + k) * DT, -0.02, i_ext=iext)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    out["split_mixed"] = {"value": n * steps / sec, "unit": UNIT, "steps": steps, "ms_per_step": 1e3 * sec / steps,
                          "note": "cm_diffusion_apply + cm_batch_step_update_act per step (two launches, "
                                  "i_ext through HBM, FP64 Vm), each call synchronising"}
    out["fused_vs_split"] = out["fused_mixed"]["value"] / out["split_mixed"]["value"]
    del b, vm, act, iext, d
    torch.cuda.empty_cache()
    return out


# Implicit finite-element leg: trilinear elements on a 128 x 128 x 64 node slab (1,048,576 nodes,
# 0.1 mm, sigma 0.1 S/m, C_m beta = 1 uF/cm^2 x 1400/cm, theta 0.5, the reference's rtol = atol =
# 1e-6). Bytes per node of one CG iteration: kernel a reads p, q, r, x, D^-1 and writes x, r, z
# (64 B); kernel b reads z, p, q, writes p, q and reads A's row: 27 entries of (4 + 8) B (364 B).
THETA_DIMS = (128, 128, 64)
THETA_ITER_BYTES = 64 + 5 * 8 + 27 * 12


def theta_leg(cm, torch, stream, args, hbm_peak, peak_kind):
    """The implicit finite-element monodomain step (acCELLerate::IntraStep with IntraRHS): TT2 mixed
    cell update + Godunov step + the solve of (C_m beta/dt M + theta K) x = (C_m beta/dt M - (1 -
    theta) K) x by Jacobi-preconditioned CG, per step; activation times."""
    from cardiomechanics_gb300 import workloads as W
    nx, ny, nz = THETA_DIMS if args.theta_dims is None else tuple(args.theta_dims)
    n = nx * ny * nz
    t0 = time.perf_counter()
    M, K = W.fe_q1_grid(nx, ny, nz)
    A, R = W.theta_operators(M, K, DT)
    del M, K
    dA, dR = cm.Diffusion(*W.csr_arrays(A)), cm.Diffusion(*W.csr_arrays(R))
    nnz_row = A.nnz / n
    del A, R
    setup_s = time.perf_counter() - t0
    th = cm.Theta(dA, dR)
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    b = cm.Batch(p, n, cm.MIXED, stream=stream.cuda_stream)
    sc = W.conductance_scales(5, n, 3, 0.95, 1.05)
    for k, h in enumerate(W.TT2_HETERO):
        b.add_hetero_value(h, p.get(h) * sc[k])
    tb = torch.tensor(np.where(np.arange(n) % nx < 3, 0.0, 1e9), device="cuda")
    vm = torch.tensor(b.init_vm(), device="cuda")
    act = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    kw = dict(textlen=1e-3, bcl=1e9, amplitude=2 * W.TT2_STIM_NA, vm_range=0.2, act_threshold=-0.02)
    b.run_theta(th, vm, 3, textbegin_per_cell=tb, act=act, **kw)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    steps = args.theta_steps
    e0.record(stream)
    st = b.run_theta(th, vm, steps, t0=3 * DT, textbegin_per_cell=tb, act=act, **kw)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    iters = st["iterations"] / max(1, st["solves"])
    # per step: the cell update (TT2 mixed, FP64 Vm in/out: 168 + 16 + 12 B), the solve's setup
    # (R and A rows, x, r, z, p, q: 2 x 27 x 12 + 6 x 8 B) and its iterations
    step_bytes = (168 + 16 + 12) + (2 * 27 * 12 + 6 * 8) + iters * THETA_ITER_BYTES
    achieved = step_bytes * n * steps / sec / 1e9
    out = {"workload": f"tt2006-epi-fe-slab-{nx}x{ny}x{nz}", "nodes": n, "nnz_per_row": nnz_row,
           "elements": "trilinear hexahedra, h 0.1 mm, sigma 0.1 S/m, C_m beta 1 uF/cm^2 x 1400/cm, theta 0.5",
           "solver": "CG + Jacobi, FP64, rtol = atol = 1e-6 (PETSc default test, preconditioned norm)",
           "value": n * steps / sec, "unit": "node-steps/s", "steps": steps, "ms_per_step": 1e3 * sec / steps,
           "cg_iterations_per_step": iters, "max_iterations": st["max_iterations"],
           "not_converged": st["not_converged"], "activated": int((act >= 0).sum().item()),
           "gpu_launches_per_step": 1 + 2 + 2 * iters + 1,
           "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                   "peak_kind": peak_kind, "bytes_per_node_step": step_bytes},
           "setup_s_host": setup_s}
    del th, dA, dR, b, vm, act, tb
    torch.cuda.empty_cache()
    return out


def precision_leg(cm, torch, stream, args, hbm_peak, peak_kind):
    """Precision form: 4,194,304 cells, the HBM-bound plain kernel (autotuned launch shape)."""
    p, b = make_batch(cm, cm.MIXED, stream.cuda_stream)
    if args.launch:
        v, g = (int(x) for x in args.launch.split(","))
        b.set_launch(v, g)
        tuned, tuned_ms = v * 100 + g, None
    else:
        tuned, tuned_ms = b.autotune(args.tune_steps)
    vm = torch.tensor(b.init_vm(), device="cuda")
    b.run(vm, 20, textbegin=0.0, textlen=1e-3, bcl=BCL, amplitude=cm_stim())
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    b.run(vm, args.mixed_steps, t0=20 * DT, textbegin=0.0, textlen=1e-3, bcl=BCL, amplitude=cm_stim())
    ev1.record(stream)
    torch.cuda.synchronize()
    sec = ev0.elapsed_time(ev1) / 1e3
    ms = 1e3 * sec / args.mixed_steps
    achieved = MIXED_BYTES_PER_CELL_STEP * N_CELLS / (ms / 1e3) / 1e9
    kernel = MIXED_KERNELS[tuned // 100] if 0 <= tuned // 100 < len(MIXED_KERNELS) else f"shape {tuned}"
    audit = b.audit()
    out = {"value": N_CELLS * args.mixed_steps / sec, "unit": UNIT, "ms_per_step": ms, "steps": args.mixed_steps,
           "workload": WORKLOAD, "cells": N_CELLS, "bcl_ms": BCL * 1e3,
           "conductance_jitter": "g_Na,g_Kr,g_K1 x U[0.9,1.1] seed 2",
           "precision": "mixed (FP32 gates/currents, compensated FP32 pairs for Vm/Na_i/K_i/CaSR)",
           "autotune": {"choice": tuned, "ms_per_step": tuned_ms}, "audit_mask": audit,
           "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                        "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                        "bytes_per_cell_step": MIXED_BYTES_PER_CELL_STEP,
                        "algorithmic_bytes_per_launch": MIXED_BYTES_PER_CELL_STEP * N_CELLS,
                        "traffic": MEASURED_TRAFFIC.get(kernel)},
           "gpu_launches": args.mixed_steps + 2}
    del b
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000, help="timed macro steps of the headline (full form)")
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--e2e-steps", type=int, default=200, help="timed C-ABI calls (one macro step each) of the end-to-end figure")
    ap.add_argument("--mixed-steps", type=int, default=2000, help="timed steps of the precision form")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", default="all",
                    choices=["all", "full", "mixed", "fp64", "surrogate", "batched", "ord", "tomek", "tissue",
                             "theta", "crn", "train"],
                    help="run one leg only (profiler captures); the contract's JSON line is printed for 'all'")
    ap.add_argument("--tune-steps", type=int, default=10)
    ap.add_argument("--crn-steps", type=int, default=500, help="timed steps of the Courtemanche mixed form")
    ap.add_argument("--crn-cells", type=int, default=CRN_CELLS, help="Courtemanche cells (fewer only for captures)")
    ap.add_argument("--fit-steps", type=int, default=2000, help="Adam steps of the training leg")
    ap.add_argument("--sur-steps", type=int, default=5000, help="timed macro steps of the 1M-cell learned form")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--multi-launch", default=None,
                    help="fixed batched launch 'tile_cells,shape,blocks_per_sm' (skips tuning; captures)")
    ap.add_argument("--batched-steps", type=int, default=640, help="timed steps of the batched form")
    ap.add_argument("--batched-instances", type=int, default=256,
                    help="instances of the batched form (fewer only for profiler captures)")
    ap.add_argument("--sur-seeds", type=int, default=3,
                    help="network seeds trained and compared on held-out cells (0: an untrained zero-output "
                         "network, for profiler captures only)")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the accuracy traces (captures only)")
    ap.add_argument("--sur-cells", type=int, default=None, help="cells of the learned leg (default 1,048,576)")
    ap.add_argument("--gen-steps", type=int, default=None,
                    help="macro steps per training population in the training leg (captures; default: all)")
    ap.add_argument("--launch", default=None, help="fixed mixed-kernel launch shape 'variant,grid_mode' (skips tuning)")
    ap.add_argument("--ord-steps", type=int, default=500,
                    help="timed steps of the O'Hara-Rudy and Tomek mixed forms")
    ap.add_argument("--ord-cells", type=int, default=ORD_CELLS,
                    help="O'Hara-Rudy and Tomek cells (fewer only for captures)")
    ap.add_argument("--no-ord", action="store_true", help="skip the O'Hara-Rudy and Tomek legs")
    ap.add_argument("--tissue-steps", type=int, default=500, help="timed steps of the coupled (tissue) leg")
    ap.add_argument("--tissue-dims", type=int, nargs=3, default=None, help="slab size (fewer nodes only for captures)")
    ap.add_argument("--no-tissue", action="store_true")
    ap.add_argument("--theta-steps", type=int, default=200, help="timed steps of the implicit FE leg")
    ap.add_argument("--theta-dims", type=int, nargs=3, default=None, help="FE slab nodes (fewer only for captures)")
    ap.add_argument("--no-theta", action="store_true")
    ap.add_argument("--tissue-model", default="tt2", choices=list(TISSUE_MODELS),
                    help="cell model of the tissue leg (the headline run uses tt2)")
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

    if args.only == "batched":
        print(json.dumps(batched_leg(cm, torch, stream, args.batched_steps, 32, hbm_peak, peak_kind,
                                     args.batched_instances, args.multi_launch)), flush=True)
        return
    if args.only == "fp64":
        _, b64 = make_batch(cm, cm.FP64, stream.cuda_stream)
        vm64 = torch.tensor(b64.init_vm(), device="cuda")
        time_device_steps(torch, cm, b64, stream, vm64, args.fp64_steps, 3, 0.0)
        return
    if args.only == "mixed":
        print(json.dumps(precision_leg(cm, torch, stream, args, hbm_peak, peak_kind)), flush=True)
        return
    if args.only == "tissue":
        print(json.dumps(tissue_leg(cm, torch, stream, args, hbm_peak, peak_kind)), flush=True)
        return
    if args.only == "theta":
        print(json.dumps(theta_leg(cm, torch, stream, args, hbm_peak, peak_kind)), flush=True)
        return
    if args.only == "crn":
        print(json.dumps(crn_leg(cm, torch, stream, args, hbm_peak, peak_kind)), flush=True)
        return
    if args.only == "train":
        print(json.dumps(training_leg(cm, torch, stream, args)), flush=True)
        return
    if args.only in ("ord", "tomek"):
        leg = "ohara_rudy" if args.only == "ord" else "tomek"
        print(json.dumps(ionic_leg(cm, torch, stream, args, hbm_peak, peak_kind, leg,
                                   cpu_seconds=0.0 if args.no_cpu else 5.0)), flush=True)
        return
    p, sur, training = train_surrogate(cm, stream, tuple(range(1, args.sur_seeds + 1)))
    if args.only == "surrogate":
        out = learned_leg(cm, torch, stream, p, sur, args.sur_steps, 20, args.sur_cells)
        out["training"] = training
        print(json.dumps(out), flush=True)
        return

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- the headline: full chosen form at scale
    full = full_form_leg(cm, torch, stream, p, sur, args.steps, args.warmup, args.e2e_steps, args.fp64_steps,
                         hbm_peak, peak_kind, barrier)
    sec = max_over_ranks(torch, full["seconds"], world)
    value = world * FULL_CELLS * SUR_SUBSTEPS * args.steps / sec
    if args.only == "full":
        if rank == 0:
            acc = headline_accuracy(full, None)
            print(json.dumps({k: v for k, v in full.items() if not k.startswith("accuracy_")} | {"accuracy": acc}),
                  flush=True)
        return
    fp32_peak = cm.fma_peak_tflops(False, stream.cuda_stream)
    fp64_peak = cm.fma_peak_tflops(True, stream.cuda_stream)
    learned = None if args.no_learned else learned_leg(cm, torch, stream, p, sur, args.sur_steps, 20)
    del sur
    torch.cuda.empty_cache()
    prec = precision_leg(cm, torch, stream, args, hbm_peak, peak_kind)
    crn = crn_leg(cm, torch, stream, args, hbm_peak, peak_kind)
    small = plain_small_leg(cm, torch, stream)
    bat = None
    if not args.no_batched:
        bat = batched_leg(cm, torch, stream, args.batched_steps, 32, hbm_peak, peak_kind)
    tissue = None if args.no_tissue else tissue_leg(cm, torch, stream, args, hbm_peak, peak_kind)
    theta = None if args.no_theta else theta_leg(cm, torch, stream, args, hbm_peak, peak_kind)
    ionic = {}
    for leg in IONIC_LEGS:
        ionic[leg] = None if args.no_ord else ionic_leg(
            cm, torch, stream, args, hbm_peak, peak_kind, leg, fp64_peak,
            cpu_seconds=5.0 if (rank == 0 and not args.no_cpu) else 0.0)
    cpu, oracle_traces = None, None
    if rank == 0 and not args.no_cpu:
        cpu, oracle_traces = cpu_baseline()
    accuracy = headline_accuracy(full, oracle_traces)

    if rank == 0:
        fp64 = full["plain_fp64"]
        fp64["fp64_fma_peak_tflops_measured"] = fp64_peak
        unmet = None if accuracy["pass"] else (
            "the network of this run misses the accuracy bars on the headline's own cells: "
            + json.dumps(accuracy["learned"]))
        line = {
            "metric": METRIC, "value": value if unmet is None else None, "unit": UNIT, "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16 (f64 audit)", "data": "synthetic",
            "config": headline_config(world),
            "accuracy": accuracy,
            "value_if_accuracy_unmet": value if unmet is not None else None,
            "value_unmet_reason": unmet,
            "coarse_only": dict(full["coarse_only"], accuracy=accuracy["coarse_only"]),
            "fallback_fraction": full["fallback_fraction"],
            "plain_fp64": fp64,
            "speedup_vs_plain_fp64": value / world / fp64["value"],
            "surrogate_stats": full["stats"],
            "training": training,
            "e2e": full["e2e"],
            "roofline": full["roofline"],
            "sur_plain_kernel": full["sur_plain_kernel"],
            "precision_form": prec,
            "plain_small": small,
            "courtemanche": crn,
            "learned_form": learned,
            "batched": bat,
            "ohara_rudy": ionic["ohara_rudy"],
            "tomek": ionic["tomek"],
            "tissue": tissue,
            "theta": theta,
            "fp32_fma_peak_tflops_measured": fp32_peak,
            "cpu_baseline": cpu,
            "gpu_launches": full["gpu_launches"],
            "clocks": full["clocks"],
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def headline_accuracy(full, oracle_traces):
    """Trace errors of the headline's network and of the coarse step alone on ACC_CELLS headline
    cells: against the oracle (the FP64 restatement of the reference Calc run on the host cores)
    when its traces exist, else against the FP64 kernel; the bars are APD90 <= 1 ms and RMS Vm
    <= 0.5 mV."""
    from cardiomechanics_gb300 import learned as L
    ph = full["accuracy_phases"]
    if oracle_traces is not None:
        ref_name = "oracle (FP64 C restatement of the reference Calc, host cores)"
        err = {k: L.trace_errors(v, oracle_traces, ph, SUR_SUBSTEPS * DT, ACC_BEATS)
               for k, v in full["accuracy_traces"].items()}
    else:
        ref_name = "plain FP64 kernel"
        err = full["accuracy_vs_fp64_kernel"]
    ok = err["learned"]["apd90_max_ms"] <= L.APD_BAR_MS and err["learned"]["rms_vm_mv_max"] <= L.RMS_BAR_MV
    return {"cells": ACC_CELLS, "beats": ACC_BEATS, "bcl_ms": FULL_BCL * 1e3, "t_end_s": ACC_T_END,
            "sample_ms": SUR_SUBSTEPS * DT * 1e3, "reference": ref_name, "cells_from": "the headline population "
            f"(seeded draw {ACC_SEED}, own conductances and phases)", "learned": err["learned"],
            "coarse_only": err["coarse_only"], "vs_fp64_kernel": full["accuracy_vs_fp64_kernel"],
            "learned_stats": full["accuracy_stats"]["learned"],
            "bars": {"apd90_ms": L.APD_BAR_MS, "rms_vm_mv": L.RMS_BAR_MV}, "pass": bool(ok)}


def cm_stim():
    from cardiomechanics_gb300 import workloads as W
    return W.TT2_STIM_NA


if __name__ == "__main__":
    main()
