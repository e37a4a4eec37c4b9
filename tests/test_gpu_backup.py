"""acCELLerate backup files through the C ABI (cm_backup_read / cm_backup_write,
acCELLerate.cpp:1511-1661) against a fixture written from the reference models' own blocks
(tests/golden/make_golden.py backup): seven nodes of three materials interleaved."""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DT = 1e-5
FIX = O.GOLDEN / "backup_mixed.abp"
# (model id, oracle model, fixture key, .ev variant)
PARTS = [(5, O.TT2, "tt2", None), (2, O.CRN, "crn", None), (12, O.ORD, "ord_endo", "endo")]
# block slots of the states (the rest are the reference's stored currents and scratch values)
STATE_SLOTS = {5: list(range(5)) + list(range(23, 36)), 2: list(range(20)) + [21], 12: [0, 1, 2, 3] + list(range(5, 42))}


def make_parts(cm, prec):
    g = np.load(O.GOLDEN / "backup_mixed.npz")
    batches, vms, ids = [], [], []
    for m, _, key, _ in PARTS:
        n = g[f"ids_{key}"].size
        b = cm.Batch(cm.Params(m, None, DT), n, prec)
        batches.append(b)
        vms.append(np.zeros(n))
        ids.append(g[f"ids_{key}"])
    return g, batches, vms, ids


@pytest.mark.parametrize("prec", [0, 1])
def test_read_fixture(gpu, prec):
    cm = gpu
    g, batches, vms, ids = make_parts(cm, prec)
    t = cm.backup_read(FIX, batches, vms, ids)
    assert t == "0.05"
    # mixed batches keep most states in FP32 (a gate at 1e-69 is 0 there)
    tol, atol = (0, 0) if prec == cm.FP64 else (1e-7, 1e-30)
    for (m, _, key, _), b, v in zip(PARTS, batches, vms):
        np.testing.assert_array_equal(v, g[f"vm_{key}"])
        blk = b.get_state(cm.LAYOUT_REF_BLOCK)
        s = STATE_SLOTS[m]
        np.testing.assert_allclose(blk[:, s], g[f"blocks_{key}"][:, s], rtol=tol, atol=atol)


def test_resume_equals_oracle(gpu, port):
    """A GPU run resumed from the backup follows the oracle resumed from the same blocks."""
    cm = gpu
    g, batches, vms, ids = make_parts(cm, cm.FP64)
    cm.backup_read(FIX, batches, vms, ids)
    for (m, om, key, var), b, v in zip(PARTS, batches, vms):
        P = port.param_vector(om, O.load_params(om, var) if var else O.load_params(om))
        T = port.tables(om, P, DT) if m != 12 else np.zeros((0, O.RTDT))
        amp = {5: W.TT2_STIM_NA, 2: W.CRN_STIM_PAPF, 12: W.ORD_STIM}[m]
        tlen = 2e-3 if m == 2 else 1e-3
        B = np.ascontiguousarray(g[f"blocks_{key}"]).copy()
        vo = g[f"vm_{key}"].copy()
        # the next beat of the fixture's protocol is at t = 1 s
        port.run(om, P, T, B, vo, 2000, DT, t0=0.05, textbegin=1.0, textlen=tlen, bcl=1.0, amp=amp)
        b.run(v, 2000, t0=0.05, textbegin=1.0, textlen=tlen, bcl=1.0, amplitude=amp)
        np.testing.assert_allclose(v, vo, rtol=0, atol=1e-9)


def test_write_round_trip(gpu, tmp_path):
    cm = gpu
    g, batches, vms, ids = make_parts(cm, cm.FP64)
    cm.backup_read(FIX, batches, vms, ids)
    out = tmp_path / "again.abp"
    cm.backup_write(out, "0.05", batches, vms, ids)
    a, b = FIX.read_bytes(), out.read_bytes()
    assert len(a) == len(b) and a[:35] == b[:35]  # the two header lines
    # node by node: Vm and the state slots as in the fixture (stored currents are zero here)
    pos = 35
    order = sorted((int(gid), k, p) for p, i in enumerate(ids) for k, gid in enumerate(i))
    for gid, k, p in order:
        m = PARTS[p][0]
        nb = cm.model_info(m).ref_block_doubles
        ra = np.frombuffer(a[pos:pos + 8 * (nb + 1)], "<f8")
        rb = np.frombuffer(b[pos:pos + 8 * (nb + 1)], "<f8")
        assert ra[0] == rb[0]
        s = [1 + x for x in STATE_SLOTS[m]]
        np.testing.assert_array_equal(ra[s], rb[s])
        pos += 8 * (nb + 1)
    assert pos == len(a)
    # consecutive parts (no node_ids) read back what they wrote
    out2 = tmp_path / "consec.abp"
    cm.backup_write(out2, "1.5", batches, vms)
    _, b2, v2, _ = make_parts(cm, cm.FP64)
    assert cm.backup_read(out2, b2, v2) == "1.5"
    for x, y, vx, vy in zip(batches, b2, vms, v2):
        np.testing.assert_array_equal(vx, vy)
        np.testing.assert_array_equal(x.get_state(), y.get_state())


def test_errors(gpu, tmp_path):
    cm = gpu
    g, batches, vms, ids = make_parts(cm, cm.FP64)
    bad = tmp_path / "bad.abp"
    data = FIX.read_bytes()
    bad.write_bytes(data[:-8])  # truncated
    with pytest.raises(cm.CMError) as e:
        cm.backup_read(bad, batches, vms, ids)
    assert e.value.code == -3
    bad.write_bytes(data.replace(b"Version1.0", b"Version2.0", 1))
    with pytest.raises(cm.CMError) as e:
        cm.backup_read(bad, batches, vms, ids)
    assert e.value.code == -3
    with pytest.raises(cm.CMError) as e:  # six nodes of parts against a seven-node file
        cm.backup_read(FIX, batches[:2] + [cm.Batch(cm.Params(12, None, DT), 1, cm.FP64)], vms[:2] + [np.zeros(1)],
                       [np.array([0, 3, 5]), np.array([1, 4]), np.array([2])])
    assert e.value.code == -3
    with pytest.raises(cm.CMError) as e:  # node 6 in two parts
        cm.backup_read(FIX, batches, vms, [ids[0], np.array([1, 6]), ids[2]])
    assert e.value.code == -1
