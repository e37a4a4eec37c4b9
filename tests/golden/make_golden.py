"""Generate the golden vectors in this folder by running the reference's own CellModel
library (compiled from the reference sources by oracle/Makefile, target `ref`).

    python tests/golden/make_golden.py [tt2] [crn] [ord] [tom] [backup]   # needs the reference tree (CM_REFERENCE_TREE)

Outputs (all seeded, deterministic):
  params_tt2_epi.json / params_crn.json  resolved parameter sets after Init + Calculate
                                         (TenTusscher2_original_Epi.ev, CourtemancheEtAl.ev)
  params_ord_<v>.json                    O'Hara-Rudy, v = endo / epi / mid (OHaraRudy_<v>.ev)
  params_tom_<v>.json                    Tomek, the same cell types (Tomek_<v>.ev)
  tables_<m>.npz    sha256 of every lookup table's bytes + every 50th row, dt = 1e-5 s
                    (TT2 and CRN; O'Hara-Rudy has none)
  step_<m>.npz      one-Calc known answers: states sampled along paced trajectories,
                    table-edge voltages, with and without stimulus (O'Hara-Rudy: one
                    file per cell type, step_ord_<v>.npz)
  trace_<m>.npz     multi-beat driver runs of jittered cells: Vm every 100 steps and the
                    final state blocks (O'Hara-Rudy: trace_ord_<v>.npz)
  backup_mixed.abp  an acCELLerate backup file of seven nodes of three models (+ .npz with the
                    parts' blocks, Vm and node indices)
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
from cardiomechanics_gb300 import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent
DT = 1e-5


def tag(model, variant=None):
    if model in (O.ORD, O.TOM):
        return f"{'ord' if model == O.ORD else 'tom'}_{variant}"
    return "tt2" if model == O.TT2 else "crn"


def hetero_names(model):
    return {O.TT2: W.TT2_HETERO, O.CRN: W.CRN_HETERO, O.ORD: W.ORD_HETERO, O.TOM: W.TOM_HETERO}[model]


def amp(model):
    return {O.TT2: W.TT2_STIM_NA, O.CRN: W.CRN_STIM_PAPF, O.ORD: W.ORD_STIM, O.TOM: W.TOM_STIM}[model]


def stim_len(model):
    """1 ms for TT2 (the workloads); Courtemanche's own GetStimTime() = 2 ms (CourtemancheEtAl.h:54);
    O'Hara-Rudy's duration parameter, 1 ms."""
    return 2e-3 if model == O.CRN else 1e-3


def ev_of(model, variant):
    return O.Ref.ev_path(model, variant) if variant else O.Ref.ev_path(model)


def dump_params(ref, model, variant=None):
    ev = ev_of(model, variant)
    cells = ref.create(model, DT, 1, ev=ev)
    p = {k: v for k, v in cells.params().items() if k}
    name = f"params_{tag(model, variant)}.json" if model in (O.ORD, O.TOM) else (
        "params_tt2_epi.json" if model == O.TT2 else "params_crn.json")
    meta = {"model": O.MODEL_NAMES[model],
            "ev_file": Path(ev).name,
            "init_vm": cells.init_vm(),
            "generator": "tests/golden/make_golden.py"}
    with open(OUT / name, "w") as f:
        json.dump({"meta": meta, "params": p}, f, indent=1, sort_keys=True)
    return p


def dump_tables(ref, port, model):
    cells = ref.create(model, DT, 1)
    names = port.table_names(model)
    digests, rows = [], []
    for n in names:
        if n == "exp250_exp50":
            t = np.zeros(O.RTDT)
            t[0], t[1] = cells.table("exp250")[0], cells.table("exp50")[0]
        else:
            t = cells.table(n)
        digests.append(hashlib.sha256(t.tobytes()).hexdigest())
        rows.append(t[::50])
    np.savez_compressed(OUT / f"tables_{tag(model)}.npz", names=np.array(names), sha256=np.array(digests),
                        rows=np.array(rows), dt=DT)


def dump_step(ref, model, variant=None):
    """States along paced trajectories of 8 jittered cells, snapshotted every 25 ms."""
    n = 8
    ev = ev_of(model, variant)
    cells = ref.create(model, DT, n, ev=ev)
    hn = hetero_names(model)
    p = cells.params()
    sc = W.conductance_scales(7, n, len(hn), 0.8, 1.2)
    for k, name in enumerate(hn):
        cells.add_hetero(name, p[name] * sc[k])
    vm = np.full(n, cells.init_vm())
    states, vms = [], []
    t = 0.0
    for chunk in range(40):  # 40 x 25 ms = 1000 ms, stimulus at t = 0
        states.append(cells.get_state())
        vms.append(vm.copy())
        cells.run(vm, 2500, DT, t0=t, textbegin=0.0, textlen=stim_len(model), bcl=1.0, amp=amp(model))
        t += 2500 * DT
    if model == O.ORD:
        # h_CaMK_fast (slot 4) is never initialised by the reference, and the stored currents
        # (slots 42..58) are not set before the first Calc; neither is read by Calc
        for s in states:
            s[:, 4] = 0.0
        states[0][:, 42:] = 0.0
    if model == O.TOM:
        # A_j, B_j (slots 4, 5) are set by the first Calc, the stored currents (48..83) too
        states[0][:, 4:6] = 0.0
        states[0][:, 48:] = 0.0
    S = np.concatenate(states)
    V = np.concatenate(vms)
    het = np.tile(sc, (1, 40))
    # table-edge voltages on rest states
    rest = states[0][:2]
    S = np.concatenate([S, rest, rest])
    V = np.concatenate([V, [-0.2000, 0.1999], [-0.1500, 0.1500]])
    het = np.concatenate([het, np.ones((len(hn), 4))], axis=1)
    m = S.shape[0]
    rng = np.random.default_rng(11)
    iext = np.where(rng.random(m) < 0.3, amp(model), 0.0)
    # one Calc per row: one reference cell per row with its own hetero values
    kat = ref.create(model, DT, m, ev=ev)
    for k, name in enumerate(hn):
        kat.add_hetero(name, p[name] * het[k])
    kat.set_state(S)
    dV = kat.calc(DT, V, iext)
    S1 = kat.get_state()
    np.savez_compressed(OUT / f"step_{tag(model, variant)}.npz", state_in=S, vm=V, i_ext=iext, hetero_names=np.array(hn),
                        hetero_scale=het, state_out=S1, dvm=dV, dt=DT)


def dump_trace(ref, model, variant=None):
    """4 jittered cells, BCL 500 ms, 2 beats, reference driver loop; Vm every 100 steps."""
    n, steps = 4, 100000
    cells = ref.create(model, DT, n, ev=ev_of(model, variant))
    hn = hetero_names(model)
    p = cells.params()
    sc = W.conductance_scales(1, n, len(hn), 0.95, 1.05)
    for k, name in enumerate(hn):
        cells.add_hetero(name, p[name] * sc[k])
    vm = np.full(n, cells.init_vm())
    tr = cells.run(vm, steps, DT, textbegin=0.0, textlen=stim_len(model), bcl=0.5, amp=amp(model), rec_every=100)
    np.savez_compressed(OUT / f"trace_{tag(model, variant)}.npz", hetero_names=np.array(hn), hetero_scale=sc,
                        n_steps=steps, dt=DT, bcl=0.5, textlen=stim_len(model), amp=amp(model), rec_every=100,
                        trace=tr, final_state=cells.get_state(), final_vm=vm)


BACKUP_VERSION = "acCELLerateBackupVersion1.0"  # acCELLerate.cpp:74


def dump_backup(ref):
    """A seven-node acCELLerate backup file with three materials interleaved (TT2 epi at nodes 0, 3,
    6; Courtemanche at 1, 4; O'Hara-Rudy endo at 2, 5), written as acCELLerate::WriteBackup does
    (acCELLerate.cpp:1616-1661: the version line, "<time> <nodes>", then per node its Vm and its
    model's GetBase() block as raw doubles), from blocks and potentials of the reference's own
    models after 50 ms of pacing. Also stores the parts' blocks, Vm and node indices."""
    parts = [(O.TT2, None, [0, 3, 6]), (O.CRN, None, [1, 4]), (O.ORD, "endo", [2, 5])]
    n_total = sum(len(ids) for _, _, ids in parts)
    rec = {}
    out = {}
    for model, variant, ids in parts:
        cells = ref.create(model, DT, len(ids), ev=ev_of(model, variant))
        vm = np.full(len(ids), cells.init_vm())
        cells.run(vm, 5000, DT, textbegin=0.0, textlen=stim_len(model), bcl=1.0, amp=amp(model))
        blk = cells.get_state()
        if model == O.ORD:
            blk[:, 4] = 0.0  # h_CaMK_fast, never set by the reference's Init
        key = tag(model, variant)
        out[f"blocks_{key}"], out[f"vm_{key}"], out[f"ids_{key}"] = blk, vm, np.array(ids, dtype=np.int64)
        for k, g in enumerate(ids):
            rec[g] = np.concatenate([[vm[k]], blk[k]]).astype("<f8").tobytes()
    with open(OUT / "backup_mixed.abp", "wb") as f:
        f.write(f"{BACKUP_VERSION}\n0.05 {n_total}\n".encode())
        for g in range(n_total):
            f.write(rec[g])
    np.savez_compressed(OUT / "backup_mixed.npz", time="0.05", **out)


def main(which):
    ref = O.Ref()
    port = O.Port()
    for model in (O.TT2, O.CRN):
        if tag(model) not in which:
            continue
        dump_params(ref, model)
        dump_tables(ref, port, model)
        dump_step(ref, model)
        dump_trace(ref, model)
        print("wrote golden vectors for", O.MODEL_NAMES[model])
    for model, key in ((O.ORD, "ord"), (O.TOM, "tom")):
        if key not in which:
            continue
        for v in O.ORD_VARIANTS:
            dump_params(ref, model, v)
            dump_step(ref, model, v)
            dump_trace(ref, model, v)
            print("wrote golden vectors for", O.MODEL_NAMES[model], v)
    if "backup" in which:
        dump_backup(ref)
        print("wrote the backup file fixture")


if __name__ == "__main__":
    main(set(sys.argv[1:]) or {"tt2", "crn", "ord", "tom", "backup"})
