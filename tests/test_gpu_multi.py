"""Batched form on the GPU: instances of uneven size and mixed model in one launch per step
give the same result (to FP32 rounding) as each instance run alone, for every launch shape and
with the CUDA-graph replay; the autotuner leaves the cells where they were."""
import numpy as np
import pytest

from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def build(cm, sizes, models, seed=5):
    out = []
    for i, (n, m) in enumerate(zip(sizes, models)):
        p = cm.Params(m, None, 1e-5)
        b = cm.Batch(p, n, cm.MIXED)
        names = W.TT2_HETERO if m == cm.TENTUSSCHER2 else W.CRN_HETERO
        sc = W.conductance_scales(seed + i, n, 3, 0.8, 1.2)
        for k, name in enumerate(names):
            b.add_hetero_value(name, p.get(name) * sc[k])
        out.append(b)
    return out


def stims(cm, models, bcl=0.3):
    rng = np.random.default_rng(3)
    return [dict(textbegin=float(rng.uniform(0, bcl)), textlen=1e-3 if m == cm.TENTUSSCHER2 else 2e-3, bcl=bcl,
                 amplitude=W.TT2_STIM_NA if m == cm.TENTUSSCHER2 else W.CRN_STIM_PAPF) for m in models]


def continued(s, n_steps, dt=1e-5):
    """The protocol after n_steps of the driver loop: t and textbegin as the driver advanced them."""
    t, tb = s.get("t0", 0.0), s["textbegin"]
    for _ in range(n_steps):
        if t >= tb and t >= tb + s["textlen"]:
            tb += s["bcl"]
        t += dt
    d = dict(s)
    d["t0"], d["textbegin"] = t, tb
    return d


def test_multi_equals_single(gpu):
    cm = gpu
    sizes = [1000, 37, 20000, 4096, 777, 65536]
    models = [cm.TENTUSSCHER2, cm.COURTEMANCHE, cm.COURTEMANCHE, cm.TENTUSSCHER2, cm.TENTUSSCHER2, cm.COURTEMANCHE]
    st = stims(cm, models)
    steps = 3000 + 7  # crosses stimuli; graph replays of 32 steps plus a remainder
    ref_b = build(cm, sizes, models)
    ref_v = []
    for b, s in zip(ref_b, st):
        v = b.init_vm()
        # same two segments as the multi below (Vm leaves the device between them)
        b.run(v, 1000, **s)
        b.run(v, steps - 1000, **continued(s, 1000))
        ref_v.append(v)
    # shapes 0-2: plain loads; 3-4: bulk-copy staged sub-tiles of 128 / 256 cells; 5-6: the same
    # as producer/consumer pipelines of 256 / 128 cells (the 1000-cell tiles of the last case are
    # not whole sub-tiles: the launcher takes the plain kernel)
    cases = [(0, 2048, 2), (1, 1024, 4), (2, 4096, 1), (3, 1024, 4), (4, 2048, 2), (3, 4096, 8), (5, 2048, 2),
             (6, 1024, 3), (5, 4096, 4), (4, 1000, 2)]
    for shape, tile, bps in cases:
        mb = build(cm, sizes, models)
        multi = cm.Multi(mb)
        multi.set_launch(tile, shape, bps)
        vms = [b.init_vm() for b in mb]
        multi.run(vms, 1000, st)
        multi.run(vms, steps - 1000, [continued(x, 1000) for x in st])
        # same per-cell code in another kernel: equal up to FP32 contraction/rounding differences
        for i in range(len(mb)):
            assert np.abs(vms[i] - ref_v[i]).max() <= 1e-6, (shape, i, np.abs(vms[i] - ref_v[i]).max())
            np.testing.assert_allclose(mb[i].get_state(), ref_b[i].get_state(), rtol=1e-4, atol=1e-7)
        assert all(b.audit() == 0 for b in mb)


def test_multi_autotune_keeps_state(gpu):
    cm = gpu
    sizes = [5000, 3000, 12000]
    models = [cm.TENTUSSCHER2, cm.COURTEMANCHE, cm.TENTUSSCHER2]
    mb = build(cm, sizes, models)
    multi = cm.Multi(mb)
    s0 = [b.get_state() for b in mb]
    choice = multi.autotune(2)
    assert choice["tile_cells"] in (1024, 2048, 4096, 8192, 16384) and choice["ms_per_step"] > 0
    for b, s in zip(mb, s0):
        assert np.array_equal(b.get_state(), s)
    vms = [b.init_vm() for b in mb]
    multi.run(vms, 64, stims(cm, models))
    assert all(np.all(np.isfinite(v)) for v in vms)


def test_multi_rejects_fp64(gpu):
    cm = gpu
    b = cm.Batch(cm.Params(5, None, 1e-5), 10, cm.FP64)
    with pytest.raises(cm.CMError) as e:
        cm.Multi([b])
    assert e.value.code == -7


def test_pipeline_shapes_with_many_instances_per_block(gpu):
    """The pipelined shapes (5-8) on 160 small instances, so that every block moves between
    instances many times and reuses its stage descriptor slots: the same cells as the
    double-buffered shape 4, and no consistency-check bit (128, 256) in any audit word."""
    cm = gpu
    rng = np.random.default_rng(11)
    sizes = [int(x) for x in rng.integers(300, 3000, 160)]
    models = [cm.TENTUSSCHER2 if i % 3 else cm.COURTEMANCHE for i in range(160)]
    st = stims(cm, models)
    out = []
    for shape, tile, bps in [(4, 1024, 1), (5, 1024, 1), (6, 1024, 1), (5, 1024, 4), (7, 1024, 2), (8, 2048, 2)]:
        mb = build(cm, sizes, models)
        multi = cm.Multi(mb)
        multi.set_launch(tile, shape, bps)
        vms = [b.init_vm() for b in mb]
        multi.run(vms, 300, st)
        assert all(b.audit() == 0 for b in mb), shape
        out.append(vms)
    for vms in out[1:]:
        for a, b in zip(vms, out[0]):
            assert np.abs(a - b).max() <= 1e-6


def test_mixed_models_against_oracle(gpu, port):
    """One batched launch per step over ten Tusscher 2006 and Courtemanche instances (own sizes,
    conductances and stimulus phases; the 3-stage 256-cell pipeline, multi_pipe_kernel<256, 3>)
    against the oracle's FP64 driver loop for each model (TenTusscher2.cpp:615-906,
    CourtemancheEtAl.cpp:85-187, CellModel.h:405-420): 3000 steps (30 ms, through each
    instance's stimulus and upstroke) in five segments, Vm compared after every segment at the
    mixed form's tolerance, and the APD-scale states after the last."""
    import oracle as O
    cm = gpu
    sizes = [4096, 2048, 1536, 3072]
    models = [cm.TENTUSSCHER2, cm.COURTEMANCHE, cm.TENTUSSCHER2, cm.COURTEMANCHE]
    st = [dict(textbegin=tb, textlen=1e-3 if m == cm.TENTUSSCHER2 else 2e-3, bcl=0.3,
               amplitude=W.TT2_STIM_NA if m == cm.TENTUSSCHER2 else W.CRN_STIM_PAPF)
          for tb, m in zip((0.0, 0.004, 0.011, 0.017), models)]
    mb = build(cm, sizes, models)
    multi = cm.Multi(mb)
    multi.set_launch(2048, 7, 2)
    vms = [b.init_vm() for b in mb]
    ref = []
    for i, (n, m) in enumerate(zip(sizes, models)):
        om = O.TT2 if m == cm.TENTUSSCHER2 else O.CRN
        P = port.param_vector(om, O.load_params(om))
        names = port.param_names(om)
        sc = W.conductance_scales(5 + i, n, 3, 0.8, 1.2)
        hn = W.TT2_HETERO if m == cm.TENTUSSCHER2 else W.CRN_HETERO
        het = {k: P[names.index(k)] * sc[j] for j, k in enumerate(hn)}
        ref.append(dict(om=om, P=P, T=port.tables(om, P, 1e-5), B=port.init_state(om, P, n),
                        v=np.full(n, port.init_vm(om, P)), het=het))
    seg, worst = 600, 0.0
    for k in range(5):
        cur = [continued(s, k * seg) for s in st]
        multi.run(vms, seg, cur)
        for i, r in enumerate(ref):
            port.run(r["om"], r["P"], r["T"], r["B"], r["v"], seg, 1e-5, t0=cur[i]["t0"],
                     textbegin=cur[i]["textbegin"], textlen=st[i]["textlen"], bcl=st[i]["bcl"],
                     amp=st[i]["amplitude"], het=r["het"], n_threads=8)
            err = float(np.abs(vms[i] - r["v"]).max())
            worst = max(worst, err)
            # FP32 gates and currents: within 1 mV through the upstroke, as the precision form
            assert err <= 1e-3, (k, i, err)
    assert all(b.audit() == 0 for b in mb)
    # slow accumulators after 30 ms, in the reference block layout: TT2 CaSR, Na_i, K_i (slots 1,
    # 3, 4, TenTusscher2.h:77); Courtemanche Ca_up, Ca_rel (slots 1, 2)
    for i, (b, r) in enumerate(zip(mb, ref)):
        cols = [1, 3, 4] if models[i] == cm.TENTUSSCHER2 else [1, 2]
        blk = b.get_state(cm.LAYOUT_REF_BLOCK).reshape(r["B"].shape)
        np.testing.assert_allclose(blk[:, cols], r["B"][:, cols], rtol=1e-3)
    print("multi vs oracle: worst |dVm|", worst * 1e3, "mV")
