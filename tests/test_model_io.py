"""Input-folder parsing with the reference's Reader.h semantics."""
import os

import numpy as np
import pytest

from lassie_gb300 import synth
from lassie_gb300.model import (InputError, load_folder, read_by_line, read_by_tab,
                                read_matrix, strtod, write_folder, compile_model)


def test_strtod_prefix_semantics():
    assert strtod("1.5e3xyz") == 1500.0
    assert strtod("  -2") == -2.0
    assert strtod("") == 0.0
    assert strtod("abc") == 0.0
    assert strtod(".5") == 0.5
    assert strtod("3\r") == 3.0


def test_reader_line_rules(tmp_path):
    p = tmp_path / "v"
    p.write_text("1\n2\n\n")          # getline: "1", "2", "" -> three values
    assert list(read_by_line(str(p))) == [1.0, 2.0, 0.0]
    p.write_text("1\t2\t\n3")         # trailing TAB adds no token
    assert list(read_by_tab(str(p))) == [1.0, 2.0, 3.0]
    p.write_text("1\t0\n0\t2\n")
    assert read_matrix(str(p)).tolist() == [[1, 0], [0, 2]]


def test_round_trip(tmp_path):
    m = synth.make_c1()
    m.cs = np.array([0, 5, 7], np.int32)
    write_folder(m, str(tmp_path))
    r = load_folder(str(tmp_path))
    assert np.array_equal(r.left, m.left) and np.array_equal(r.right, m.right)
    assert np.array_equal(r.k, m.k) and np.array_equal(r.x0, m.x0)
    assert np.array_equal(r.t, m.t) and list(r.cs) == [0, 5, 7]


def test_missing_mandatory(tmp_path):
    m = synth.tiny_network("decay")
    write_folder(m, str(tmp_path))
    os.remove(tmp_path / "c_vector")
    with pytest.raises(InputError) as e:
        load_folder(str(tmp_path))
    assert e.value.code == -4


def test_stochastic_conversion(tmp_path):
    m = synth.tiny_network("bimolecular")
    write_folder(m, str(tmp_path))
    (tmp_path / "modelkind").write_text("stochastic\n")
    (tmp_path / "volume").write_text("1e-15\n")
    r = load_folder(str(tmp_path))
    conv = 1e-15 * 6.022e23
    assert r.k[0] == pytest.approx(m.k[0] * conv)
    assert r.x0[0] == pytest.approx(m.x0[0] / conv)


def test_bad_modelkind(tmp_path):
    write_folder(synth.tiny_network("decay"), str(tmp_path))
    (tmp_path / "modelkind").write_text("banana\n")
    with pytest.raises(InputError) as e:
        load_folder(str(tmp_path))
    assert e.value.code == -7


def test_compile_model_orders():
    m = synth.make_c1()
    cm = compile_model(m.left, m.right)
    for i in range(cm.n_species):
        rows = cm.sp_rxn[cm.sp_ptr[i]:cm.sp_ptr[i + 1]]
        assert np.all(np.diff(rows) > 0)
    for j in range(cm.n_reactions):
        sp = cm.rxn_species[cm.rxn_ptr[j]:cm.rxn_ptr[j + 1]]
        assert np.all(np.diff(sp) > 0)


def test_synthetic_powers_are_correctly_rounded():
    """10^u and exp(x) of the generators are correctly rounded (checked
    against 50-digit decimal arithmetic), so a seed gives the same network on
    every machine."""
    from decimal import Decimal, getcontext
    from lassie_gb300 import synth
    getcontext().prec = 50
    rng = np.random.default_rng(11)
    u = np.concatenate([rng.uniform(-8, 8, 3000), [-6.0, -4.0, 0.0, 0.5, 2.0, 6.0]])
    want = np.array([float(Decimal(10) ** Decimal(x)) for x in u])
    assert np.array_equal(synth.pow10(u), want)
    x = np.concatenate([rng.normal(0, 3, 3000), [0.0, -1.0, 1.0]])
    want = np.array([float(Decimal(v).exp()) for v in x])
    assert np.array_equal(synth.exp_rn(x), want)
