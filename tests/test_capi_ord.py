"""Host side of the O'Hara-Rudy model in libcmgb300.so (no GPU): the built-in parameter set
equals the reference's OHaraRudy.ev after Calculate(), .ev files of the other cell types load,
and the model's layouts are the reference's."""
import numpy as np
import pytest

import oracle as O

ORD = 12


def write_ev(path, values):
    with open(path, "w") as f:
        f.write(f"CELLMODEL*IBT*KA\nOHaraRudy\n{len(values)}\n")
        for k, v in values.items():
            f.write(f"{k} {v!r}\n")


def base_values(cmlib, variant):
    ref = O.load_params(O.ORD, variant)
    p = cmlib.Params(ORD, None, 1e-5)
    names = [n for n in ref if n not in ("",)]
    base = {}
    for n in names:
        try:
            p.set(n, ref[n])
            base[n] = ref[n]
        except cmlib.CMError as e:
            assert "derived" in str(e), n  # derived values are recomputed, not read
    return base


def test_builtin_parameters_equal_reference_endo(cmlib):
    p = cmlib.Params(ORD, None, 1e-5)
    ref = O.load_params(O.ORD, "endo")
    for name, v in ref.items():
        assert p.get(name) == v, name
    assert p.info.n_tables == 0 and p.info.n_state_vars == 41 and p.info.ref_block_doubles == 59


@pytest.mark.parametrize("variant", ["epi", "mid"])
def test_ev_files_of_other_cell_types(cmlib, tmp_path, variant):
    base = base_values(cmlib, variant)
    assert len(base) == 81  # the entry count of the reference's OHaraRudy_*.ev files
    path = tmp_path / f"OHaraRudy_{variant}.ev"
    write_ev(path, base)
    p = cmlib.Params(ORD, str(path), 1e-5)
    for name, v in O.load_params(O.ORD, variant).items():
        assert p.get(name) == v, name


def test_ev_missing_entry_is_an_error(cmlib, tmp_path):
    base = base_values(cmlib, "endo")
    del base["IKr_Multiplier"]
    path = tmp_path / "bad.ev"
    write_ev(path, base)
    with pytest.raises(cmlib.CMError) as e:
        cmlib.Params(ORD, str(path), 1e-5)
    assert e.value.code == -4 and "IKr_Multiplier" in str(e.value)


def test_layouts(cmlib):
    names = cmlib.state_names(ORD)
    assert len(names) == 41 and "h_CaMK_fast" not in names
    assert names[:4] == ["m", "h_fast", "h_slow", "j"] and names[4] == "h_CaMK_slow" and names[-1] == "Ca_TRPN"
    p = cmlib.Params(ORD, None, 1e-5)
    assert p.info.amplitude == -50.0 and p.info.stim_time == 0.001
    with pytest.raises(cmlib.CMError):
        p.table("m_inf")
