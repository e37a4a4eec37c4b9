"""Generate the golden vectors in this folder by running the reference's own CellModel
library (compiled from the reference sources by oracle/Makefile, target `ref`).

    python tests/golden/make_golden.py            # needs the reference tree (CM_REFERENCE_TREE)

Outputs (all seeded, deterministic):
  params_tt2_epi.json / params_crn.json  resolved parameter sets after Init + Calculate
                                         (TenTusscher2_original_Epi.ev, CourtemancheEtAl.ev)
  tables_<m>.npz    sha256 of every lookup table's bytes + every 50th row, dt = 1e-5 s
  step_<m>.npz      one-Calc known answers: states sampled along paced trajectories,
                    table-edge voltages, with and without stimulus
  trace_<m>.npz     multi-beat driver runs of jittered cells: Vm every 100 steps and the
                    final state blocks
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


def tag(model):
    return "tt2" if model == O.TT2 else "crn"


def hetero_names(model):
    return W.TT2_HETERO if model == O.TT2 else W.CRN_HETERO


def amp(model):
    return W.TT2_STIM_NA if model == O.TT2 else W.CRN_STIM_PAPF


def stim_len(model):
    """1 ms for TT2 (the workloads); Courtemanche's own GetStimTime() = 2 ms (CourtemancheEtAl.h:54)."""
    return 1e-3 if model == O.TT2 else 2e-3


def dump_params(ref, model):
    cells = ref.create(model, DT, 1)
    p = {k: v for k, v in cells.params().items() if k}
    name = "params_tt2_epi.json" if model == O.TT2 else "params_crn.json"
    meta = {"model": O.MODEL_NAMES[model],
            "ev_file": Path(O.Ref.ev_path(model)).name,
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


def dump_step(ref, model):
    """States along paced trajectories of 8 jittered cells, snapshotted every 25 ms."""
    n = 8
    cells = ref.create(model, DT, n)
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
    kat = ref.create(model, DT, m)
    for k, name in enumerate(hn):
        kat.add_hetero(name, p[name] * het[k])
    kat.set_state(S)
    dV = kat.calc(DT, V, iext)
    S1 = kat.get_state()
    np.savez_compressed(OUT / f"step_{tag(model)}.npz", state_in=S, vm=V, i_ext=iext, hetero_names=np.array(hn),
                        hetero_scale=het, state_out=S1, dvm=dV, dt=DT)


def dump_trace(ref, model):
    """4 jittered cells, BCL 500 ms, 2 beats, reference driver loop; Vm every 100 steps."""
    n, steps = 4, 100000
    cells = ref.create(model, DT, n)
    hn = hetero_names(model)
    p = cells.params()
    sc = W.conductance_scales(1, n, len(hn), 0.95, 1.05)
    for k, name in enumerate(hn):
        cells.add_hetero(name, p[name] * sc[k])
    vm = np.full(n, cells.init_vm())
    tr = cells.run(vm, steps, DT, textbegin=0.0, textlen=stim_len(model), bcl=0.5, amp=amp(model), rec_every=100)
    np.savez_compressed(OUT / f"trace_{tag(model)}.npz", hetero_names=np.array(hn), hetero_scale=sc,
                        n_steps=steps, dt=DT, bcl=0.5, textlen=stim_len(model), amp=amp(model), rec_every=100,
                        trace=tr, final_state=cells.get_state(), final_vm=vm)


def main():
    ref = O.Ref()
    port = O.Port()
    for model in (O.TT2, O.CRN):
        dump_params(ref, model)
        dump_tables(ref, port, model)
        dump_step(ref, model)
        dump_trace(ref, model)
        print("wrote golden vectors for", O.MODEL_NAMES[model])


if __name__ == "__main__":
    main()
