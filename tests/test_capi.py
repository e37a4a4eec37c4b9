"""C-ABI library on the host: it loads, exports every symbol include/*.h declares, its
parameter sets and FP64 tables equal the reference's, and it refuses bad input. No kernel
is launched here."""
import hashlib
import re

import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import analysis as A
from cardiomechanics_gb300 import workloads as W

ROOT = O.HERE.parent
TAG = {5: "tt2", 2: "crn"}
ORACLE_MODEL = {5: O.TT2, 2: O.CRN}


def declared_symbols():
    syms = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        syms |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(cm_\w+)\s*\(", text, flags=re.M))
    return syms


def test_exports_every_declared_symbol(cmlib):
    L = cmlib.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing
    assert set(cmlib.ABI_SYMBOLS) <= syms


def test_abi_version_and_models(cmlib):
    L = cmlib.lib()
    assert L.cm_abi_version() == 1
    assert L.cm_model_from_name(b"TenTusscher2") == 5
    assert L.cm_model_from_name(b"CourtemancheEtAl") == 2
    assert L.cm_model_from_name(b"OHaraRudy") == 12
    assert L.cm_model_from_name(b"Tomek") == 14
    assert L.cm_model_from_name(b"OHaraRudyIso") == -1
    assert cmlib.model_info(5).ref_block_doubles == 36
    assert cmlib.model_info(2).ref_block_doubles == 22
    assert cmlib.model_info(12).ref_block_doubles == 59
    assert cmlib.model_info(14).ref_block_doubles == 84
    assert cmlib.state_names(5)[:5] == ["Ca_i", "CaSR", "CaSS", "Na_i", "K_i"]
    with pytest.raises(cmlib.CMError):
        cmlib.model_info(13)


@pytest.mark.parametrize("model", [5, 2])
def test_builtin_parameters_equal_reference(cmlib, model):
    p = cmlib.Params(model, None, 1e-5)
    ref = O.load_params(ORACLE_MODEL[model])
    checked = 0
    for name, v in ref.items():
        try:
            got = p.get(name)
        except cmlib.CMError:
            continue
        assert got == v, name
        checked += 1
    assert checked > 100


@pytest.mark.parametrize("model", [5, 2])
def test_tables_bitwise_reference(cmlib, model):
    g = np.load(O.GOLDEN / f"tables_{TAG[model]}.npz")
    p = cmlib.Params(model, None, float(g["dt"]))
    for name, sha, rows in zip(g["names"], g["sha256"], g["rows"]):
        name = str(name)
        if name == "exp250_exp50":
            t = np.zeros(4000)
            t[0], t[1] = p.table("exp250")[0], p.table("exp50")[0]
        else:
            t = p.table(name)
        if hashlib.sha256(t.tobytes()).hexdigest() != sha:
            np.testing.assert_allclose(t[::50], rows, rtol=4e-15, err_msg=name)


def write_ev(path, model_name, values, count=None, magic="CELLMODEL*IBT*KA"):
    items = list(values.items())
    with open(path, "w") as f:
        f.write(f"# generated\n{magic}\n{model_name}\n{count if count is not None else len(items)}\n")
        for k, v in items:
            f.write(f"{k} {v!r}\n")
            if k == "R":
                f.write("# a comment line between entries\n\n")


@pytest.mark.parametrize("model", [5, 2])
def test_ev_file_roundtrip(cmlib, tmp_path, model):
    name = "TenTusscher2" if model == 5 else "CourtemancheEtAl"
    ref = O.load_params(ORACLE_MODEL[model])
    p0 = cmlib.Params(model, None, 1e-5)
    vals = {k: v for k, v in ref.items() if not k.startswith("UNDEF")}
    vals["g_Na"] = vals["g_Na"] * 0.5
    path = tmp_path / "m.ev"
    write_ev(path, name, vals)
    p = cmlib.Params(model, str(path), 1e-5)
    assert p.get("g_Na") == vals["g_Na"]
    assert p.get("K_o") == p0.get("K_o")


def test_ev_file_errors(cmlib, tmp_path):
    ref = O.load_params(O.TT2)
    path = tmp_path / "bad.ev"
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Params(5, str(tmp_path / "missing.ev"), 1e-5)
    assert e.value.code == -3
    write_ev(path, "TenTusscher2", ref, magic="CELLMODEL*XXX*KA")
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Params(5, str(path), 1e-5)
    assert e.value.code == -3
    write_ev(path, "CourtemancheEtAl", ref)
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Params(5, str(path), 1e-5)
    assert e.value.code == -3
    partial = {k: v for k, v in ref.items() if k != "g_Kr"}
    write_ev(path, "TenTusscher2", partial)
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Params(5, str(path), 1e-5)
    assert e.value.code == -4 and "g_Kr" in str(e.value)
    write_ev(path, "TenTusscher2", ref, count=300)
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Params(5, str(path), 1e-5)
    assert e.value.code == -3


def test_params_set_rebuilds_tables(cmlib):
    p = cmlib.Params(5, None, 1e-5)
    t0 = p.table("rec_ipK").copy()
    p.set("g_pK", 2 * p.get("g_pK"))
    np.testing.assert_allclose(p.table("rec_ipK"), 2 * t0, rtol=1e-15)
    p.set("K_o", 6.0)
    assert p.get("RTONF") > 0
    with pytest.raises(cmlib.CMError):
        p.set("RTONF", 1.0)  # derived
    with pytest.raises(cmlib.CMError):
        p.get("no_such_parameter")
    with pytest.raises(cmlib.CMError):
        cmlib.Params(5, None, -1.0)


def test_dt_changes_tables(cmlib, port):
    for dt in (1e-5, 2.5e-5):
        p = cmlib.Params(5, None, dt)
        P = port.param_vector(O.TT2, O.load_params(O.TT2))
        T = port.tables(O.TT2, P, dt)
        k = port.table_names(O.TT2).index("exptau_m")
        assert np.array_equal(p.table("exptau_m"), T[k])


def test_no_cpu_fallback(cmlib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = cmlib.Params(5, None, 1e-5)
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Batch(p, 16)
    assert e.value.code == -5


def test_workload_rng_is_counter_based():
    a = W.conductance_scales(1, 1000, 3, 0.95, 1.05)
    b = W.conductance_scales(1, 1000, 3, 0.95, 1.05, cells=np.arange(500, 1000))
    assert np.array_equal(a[:, 500:], b)
    assert a.min() >= 0.95 and a.max() <= 1.05
    assert abs(a.mean() - 1.0) < 0.005
    assert not np.array_equal(a, W.conductance_scales(2, 1000, 3, 0.95, 1.05))


def test_ap_markers_on_synthetic_trace():
    dt = 1e-4
    t = np.arange(0, 0.5, dt)
    # piecewise-linear AP: rest -0.085, upstroke 5..6 ms to +0.03, plateau, linear repolarisation 200..300 ms
    v = np.full_like(t, -0.085)
    up = (t >= 0.005) & (t < 0.006)
    v[up] = -0.085 + (t[up] - 0.005) / 0.001 * 0.115
    v[(t >= 0.006) & (t < 0.2)] = 0.03
    rp = (t >= 0.2) & (t < 0.3)
    v[rp] = 0.03 - (t[rp] - 0.2) / 0.1 * 0.115
    tu, apd, vp = A.ap_markers(v[None, :], dt, 0.0)
    assert abs(tu[0] - (0.005 + 0.065 / 0.115 * 0.001)) < 1e-9
    v90 = 0.03 - 0.9 * 0.115
    t90 = 0.2 + (0.03 - v90) / 0.115 * 0.1
    assert abs(apd[0] - (t90 - tu[0])) < 1e-9
    tu2, apd2, _ = A.ap_markers(np.full((1, 100), -0.08), dt, 0.0)
    assert np.isnan(tu2[0]) and np.isnan(apd2[0])


def test_print_columns(cmlib):
    """Print / LongPrint column names of the four models, in the reference's order and count
    (GetParameterNames / GetLongParameterNames): the per-node view and GetResVal rely on them."""
    import ctypes
    L = cmlib.lib()
    want = {5: (19, 17, "m", "I_tot"), 2: (21, 19, "m", "I_SAC"), 12: (41, 17, "m", "I_SAC"),
            14: (48, 33, "m", "I_SAC")}
    for model, (n_short, n_long, first, last) in want.items():
        assert L.cm_model_print_names(model, 0, None, 0) == n_short
        n = L.cm_model_print_names(model, 1, None, 0)
        assert n == n_short + n_long
        names = (ctypes.c_char_p * n)()
        assert L.cm_model_print_names(model, 1, names, n) == n
        got = [x.decode() for x in names]
        assert got[0] == first and got[-1] == last and len(set(got)) == n, (model, got)
    assert L.cm_model_print_names(13, 0, None, 0) < 0
