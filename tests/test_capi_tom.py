"""Host side of the Tomek model in libcmgb300.so (no GPU): the built-in parameter set equals
the reference's Tomek.ev after Calculate(), .ev files of the other cell types load, and the
model's layouts are the reference's."""
import numpy as np
import pytest

import oracle as O

TOM = 14


def write_ev(path, values):
    with open(path, "w") as f:
        f.write(f"CELLMODEL*IBT*KA\nTomek\n{len(values)}\n")
        for k, v in values.items():
            f.write(f"{k} {v!r}\n")


def base_values(cmlib, variant):
    ref = O.load_params(O.TOM, variant)
    p = cmlib.Params(TOM, None, 1e-5)
    base = {}
    for n in ref:
        try:
            p.set(n, ref[n])
            base[n] = ref[n]
        except cmlib.CMError as e:
            assert "derived" in str(e), n  # derived values are recomputed, not read
    return base


def test_builtin_parameters_equal_reference_endo(cmlib):
    p = cmlib.Params(TOM, None, 1e-5)
    ref = O.load_params(O.TOM, "endo")
    for name, v in ref.items():
        assert p.get(name) == v, name
    assert p.info.n_tables == 0 and p.info.n_state_vars == 44 and p.info.ref_block_doubles == 84
    assert cmlib.lib().cm_model_from_name(b"Tomek") == TOM


@pytest.mark.parametrize("variant", ["epi", "mid"])
def test_ev_files_of_other_cell_types(cmlib, tmp_path, variant):
    base = base_values(cmlib, variant)
    assert len(base) == 78  # the entry count of the reference's Tomek_*.ev files
    path = tmp_path / f"Tomek_{variant}.ev"
    write_ev(path, base)
    p = cmlib.Params(TOM, str(path), 1e-5)
    for name, v in O.load_params(O.TOM, variant).items():
        assert p.get(name) == v, name


def test_ev_missing_entry_is_an_error(cmlib, tmp_path):
    base = base_values(cmlib, "endo")
    del base["Cl_o"]
    path = tmp_path / "bad.ev"
    write_ev(path, base)
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Params(TOM, str(path), 1e-5)
    assert e.value.code == -4 and "Cl_o" in str(e.value)


def test_layouts(cmlib):
    names = cmlib.state_names(TOM)
    assert len(names) == 44
    assert not {"A_h", "B_h", "A_j", "B_j"} & set(names)
    assert names[:3] == ["m", "h", "j"] and "Cl_i" in names and names[-1] == "Ca_TRPN"
    p = cmlib.Params(TOM, None, 1e-5)
    assert p.info.amplitude == -53.0 and p.info.stim_time == 0.001
    with pytest.raises(cmlib.CMError):
        p.table("m_inf")


def test_init_state_is_the_references(cmlib, port):
    """Init_<name> for every state, troponin as a fraction of 0.07 (Tomek.cpp:55-107)."""
    P = port.param_vector(O.TOM, O.load_params(O.TOM, "endo"))
    B = port.init_state(O.TOM, P, 1)[0]
    blk = [0, 3, 6] + list(range(7, 48))  # block slot of each SOA state
    p = cmlib.Params(TOM, None, 1e-5)
    s = np.array([p.get("Init_" + n) for n in cmlib.state_names(TOM)[:-1]] + [p.get("Init_Ca_TRPN") / 0.07])
    np.testing.assert_array_equal(s, B[blk])
