"""Training, selection and trace checks of the learned macro step (ten Tusscher 2006).

The surrogate (cm_surrogate_*) is trained on trajectories of the plain integrator and judged,
like the precision form, by whole-trace errors against FP64 runs: APD90, upstroke time and RMS
Vm over several beats (definitions in `analysis`).

Training data (`generate`): three populations of 2048 cells with g_Na, g_Kr, g_K1 x U[0.85,
1.15], every k-th cell sampled at every macro step outside the stimulus and the upstroke:
  * BCL 500 ms with the first stimulus at 490 ms -- the rest from the initial state that a cell
    whose pacing starts late spends (per-cell stimulus phases leave cells at rest for up to one
    cycle), then five beats;
  * BCL 800 ms, three beats; BCL 1000 ms, two beats.
Data from one protocol only (all cells stimulated at t = 0) left the initial rest outside the
training set, and the network's Vm and concentration corrections there drifted by several mV
within 20-60 ms; gate corrections alone stayed accurate.

Selection (`train_and_select`): one dataset, several network seeds (deterministic: the same
seed gives the same network), and for each network three correction sets -- all 19 outputs,
all but Vm, the 13 gates -- whose corrections are applied (the others keep the coarse step's
value). Each candidate runs a selection population (per-cell phases, BCL 500 ms) and is scored
by its worse error relative to the bars (APD90 / 1 ms, RMS Vm / 0.5 mV) against the FP64 kernel
on the same cells; the lowest score is kept. The selection cells are never the cells a caller
checks accuracy on afterwards.
"""
from __future__ import annotations

import time

import numpy as np

from . import analysis as A
from . import workloads as W

DT = 1e-5
SUBSTEPS = 10
BCL = 0.5
# (population seed, BCL [s], first stimulus [s], simulated time [s], cell stride)
TRAINING = ((11, 0.5, 0.49, 2.99, 4), (12, 0.8, 0.0, 2.4, 6), (13, 1.0, 0.0, 2.0, 8))
TRAINING_CELLS = 2048
MAX_PAIRS = 30_000_000
CORRECTION_SETS = {"all": tuple(range(19)), "no_vm": tuple(range(1, 19)), "gates": tuple(range(1, 14))}
APPLIED = slice(63, 82)  # the blob's applied correction scales (cm_surrogate_get_blob)
OUTPUT_NAMES = ("Vm", "m", "h", "j", "xr1", "xr2", "xs", "r", "s", "d", "f", "f2", "fCa", "Rq", "Ca_i", "CaSS",
                "CaSR", "Na_i", "K_i")
SELECTION = dict(cells=128, het_seed=41, phase_seed=42, t_end=2.5, sample_macro=10)
APD_BAR_MS, RMS_BAR_MV = 1.0, 0.5


def _stream(stream):
    return None if stream is None else stream.cuda_stream


def population(cm, p, n, het_seed, precision, stream=None, cells=None):
    """n cells with g_Na, g_Kr, g_K1 x U[0.85, 1.15] drawn for cell indices `cells` of stream
    het_seed (default 0..n-1)."""
    b = cm.Batch(p, n, precision, stream=_stream(stream))
    sc = W.conductance_scales(het_seed, n, 3, 0.85, 1.15, cells=cells)
    for k, name in enumerate(W.TT2_HETERO):
        b.add_hetero_value(name, p.get(name) * sc[k])
    return b


def generate(cm, p, sur, stream=None, max_macro=None):
    """Training pairs of the populations in TRAINING; returns the number of pairs held.
    max_macro caps the macro steps per population (profiler captures only)."""
    n = 0
    for seed, bcl, tb, t_end, stride in TRAINING:
        b = population(cm, p, TRAINING_CELLS, seed, cm.MIXED, stream)
        v = b.init_vm()
        n_macro = int(round(t_end / (SUBSTEPS * DT)))
        if max_macro is not None:
            n_macro = min(n_macro, max_macro)
        n = sur.generate(b, v, n_macro, textbegin=tb, textlen=1e-3, bcl=bcl, amplitude=W.TT2_STIM_NA,
                         cell_stride=stride, max_pairs=MAX_PAIRS)
    return n


def fit(sur, seed):
    """A fresh network from seed, 6000 Adam steps at 1e-3 then 4000 at 3e-4 (minibatch seeds
    derived from seed); returns the final normalised loss."""
    sur.reset_network(seed)
    sur.fit(batch=4096, steps=6000, lr=1e-3, seed=2 * seed + 1)
    return sur.fit(batch=8192, steps=4000, lr=3e-4, seed=2 * seed + 2)


def with_corrections(blob, outputs):
    """The blob with corrections applied only to `outputs` (indices into OUTPUT_NAMES)."""
    out = np.array(blob, np.float32, copy=True)
    keep = np.zeros(19, bool)
    keep[list(outputs)] = True
    out[APPLIED] = np.where(keep, out[APPLIED], 0.0)
    return out


def fp64_traces(cm, p, n, het_seed, phases, t_end, sample_macro, stream=None, cells=None):
    """Vm of n cells run by the plain FP64 kernel (the reference arithmetic) with per-cell first
    stimulus times `phases` at BCL 500 ms, sampled every sample_macro macro steps from t = 0."""
    import torch
    b = population(cm, p, n, het_seed, cm.FP64, stream, cells)
    vm = torch.tensor(b.init_vm(), device="cuda")
    tbc = torch.tensor(np.asarray(phases, np.float64), device="cuda")
    every = sample_macro * SUBSTEPS
    n_steps = int(round(t_end / DT))
    return b.run(vm, n_steps + 1, textlen=1e-3, bcl=BCL, amplitude=W.TT2_STIM_NA, textbegin_per_cell=tbc,
                 probe_cells=np.arange(n), probe_every=every)


def surrogate_traces(cm, p, sur, n, het_seed, phases, t_end, sample_macro, mode, stream=None, cells=None,
                     audit_mod=100):
    """The same cells advanced by the learned macro step (mode: cm_batch_run_surrogate bits);
    returns (traces sampled like fp64_traces, summed statistics)."""
    import torch
    b = population(cm, p, n, het_seed, cm.MIXED, stream, cells)
    vm = torch.tensor(b.init_vm(), device="cuda")
    tbc = torch.tensor(np.asarray(phases, np.float64), device="cuda")
    n_rec = int(round(t_end / DT)) // (sample_macro * SUBSTEPS) + 1
    tr = torch.zeros((n_rec, n), dtype=torch.float64, device="cuda")
    tr[0] = vm
    t = 0.0
    tot = {"surrogate": 0, "fallback": 0, "cell_macro_steps": 0, "max_audit_err_mv": 0.0}
    for k in range(1, n_rec):
        st = b.run_surrogate(sur, vm, sample_macro, t0=t, textbegin_per_cell=tbc, textlen=1e-3, bcl=BCL,
                             amplitude=W.TT2_STIM_NA, mode=mode, audit_mod=audit_mod)
        for _ in range(sample_macro * SUBSTEPS):
            t += DT
        tr[k] = vm
        for key in ("surrogate", "fallback", "cell_macro_steps"):
            tot[key] += int(st[key])
        tot["max_audit_err_mv"] = max(tot["max_audit_err_mv"], float(st["max_audit_err_mv"]))
    return tr.T.cpu().numpy(), tot


def trace_errors(tr, ref, phases, dt_sample, beats):
    """Largest APD90 and upstroke-time errors [ms] over `beats` beats per cell, largest per-cell
    RMS and absolute Vm errors [mV], against the reference traces on the same samples."""
    m = min(tr.shape[1], ref.shape[1])
    tr, ref = tr[:, :m], ref[:, :m]
    # one stimulus more than the beats counted: each counted beat's window ends at the next
    # stimulus, never in the following action potential
    ts = np.array([np.asarray(phases) + k * BCL for k in range(beats + 1)])
    u, a = A.beat_markers(tr, dt_sample, ts)
    uo, ao = A.beat_markers(ref, dt_sample, ts)
    u, a, uo, ao = u[:beats], a[:beats], uo[:beats], ao[:beats]
    d = np.abs(tr - ref) * 1e3
    missing = int((np.isnan(a) & ~np.isnan(ao)).sum())  # beats the reference has and this trace lacks
    apd = np.abs(a - ao)
    rms = np.sqrt((d ** 2).mean(axis=1))
    return {"apd90_max_ms": float(np.nanmax(apd) * 1e3) if missing == 0 else float("inf"),
            "apd90_mean_ms": float(np.nanmean(apd) * 1e3),
            "upstroke_max_ms": float(np.nanmax(np.abs(u - uo)) * 1e3),
            "rms_vm_mv_max": float(rms.max()), "rms_vm_mv_mean": float(rms.mean()),
            "max_abs_vm_mv": float(d.max()), "missing_beats": missing, "cells": int(tr.shape[0]), "beats": beats}


def score(err):
    """The worse of the two bars' fractions (APD90 / 1 ms, RMS Vm / 0.5 mV): <= 1 meets both."""
    return max(err["apd90_max_ms"] / APD_BAR_MS, err["rms_vm_mv_max"] / RMS_BAR_MV)


def selection_phases(n=SELECTION["cells"], seed=SELECTION["phase_seed"]):
    return W.uniform(seed, np.arange(n, dtype=np.uint64)) * BCL


def train_and_select(cm, p, sur, seeds=(1, 2, 3), stream=None, log=None):
    """Generates the dataset, trains one network per seed, scores every (seed, correction set)
    on the selection population and leaves the best candidate in `sur`. Returns a report."""
    t0 = time.perf_counter()
    pairs = generate(cm, p, sur, stream)
    t_gen = time.perf_counter() - t0
    sel = SELECTION
    ph = selection_phases()
    dt_s = sel["sample_macro"] * SUBSTEPS * DT
    beats = int(np.floor((sel["t_end"] - ph.max()) / BCL))
    ref = fp64_traces(cm, p, sel["cells"], sel["het_seed"], ph, sel["t_end"], sel["sample_macro"], stream)
    coarse_tr, _ = surrogate_traces(cm, p, sur, sel["cells"], sel["het_seed"], ph, sel["t_end"], sel["sample_macro"],
                                    cm.SUR_COARSE_ONLY, stream)
    coarse = trace_errors(coarse_tr, ref, ph, dt_s, beats)
    candidates = []
    best = None
    t_fit = 0.0
    for seed in seeds:
        t1 = time.perf_counter()
        loss = fit(sur, seed)
        t_fit += time.perf_counter() - t1
        blob = sur.get_blob()
        for name, outs in CORRECTION_SETS.items():
            cand = with_corrections(blob, outs)
            sur.set_blob(cand)
            tr, _ = surrogate_traces(cm, p, sur, sel["cells"], sel["het_seed"], ph, sel["t_end"], sel["sample_macro"],
                                     0, stream)
            err = trace_errors(tr, ref, ph, dt_s, beats)
            c = {"seed": seed, "corrections": name, "loss": float(loss), "score": score(err), **err}
            candidates.append(c)
            if log:
                log(c)
            if best is None or c["score"] < best[0]["score"]:
                best = (c, cand)
    sur.set_blob(best[1])
    return {"pairs": int(pairs), "generate_s": t_gen, "fit_s": t_fit, "seconds": time.perf_counter() - t0,
            "selected": best[0], "coarse_only": {**coarse, "score": score(coarse)}, "candidates": candidates,
            "selection": {"cells": sel["cells"], "t_end_s": sel["t_end"], "bcl_ms": BCL * 1e3,
                          "sample_ms": dt_s * 1e3, "beats": beats, "reference": "plain FP64 kernel"}}
