"""The drop-in CLI end to end on the GPU: a LASSIE input folder in, the
reference's output files out, trajectories equal to the oracle's."""
import os
import subprocess

import numpy as np
import pytest

from lassie_gb300 import build, synth
from lassie_gb300.model import write_folder
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def read_table(path):
    rows = []
    with open(path) as f:
        for line in f:
            vals = [float(v) for v in line.strip().split("\t") if v != ""]
            if vals:
                rows.append(vals)
    return np.asarray(rows)


@pytest.mark.parametrize("engine", ["fp64", "mixed"])
def test_cli_outputs(gpu, tmp_path, engine):
    build.build()
    # instance 35: backward-Euler steps and one RKF45 step, and its trajectory
    # is insensitive to last-bit differences of the linear solve
    m = synth.shorten(synth.make_c4_instance(35), 1.0, 11)
    m.cs = np.array([0, 3, 17, 40], np.int32)
    inp, out = tmp_path / "in", tmp_path / "out"
    write_folder(m, str(inp))
    r = subprocess.run([build.CLI, str(inp), str(out), "-engine", engine, "-root", "sqrt",
                        "-dump-f64", "-stats"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Total running time" in r.stdout
    ref, _, rc = O.solve(m)
    full = read_table(out / "output" / "Solution.f64")
    assert np.array_equal(full[:, 0], m.t)
    if engine == "fp64":
        assert np.array_equal(full[:, 1:], ref)
    else:
        assert np.all(np.abs(full[:, 1:] - ref) <= 1e-9 + 1e-6 * np.abs(ref))
    sol = read_table(out / "output" / "Solution")
    assert sol.shape == (11, 5)
    assert np.allclose(sol[:, 1:], ref, rtol=1e-4)  # %.4e text
    with open(out / "output" / "SpeciesSampling") as f:
        assert f.read() == "Saving species' dynamics: \n0; 3; 17; 40; \n"
    prog = (out / "output" / "ProgressSimulation").read_text().split()
    assert float(prog[-1]) == 1.0
    assert os.path.exists(out / "output" / "infoBlockThread")


def test_cli_bdf_controller(gpu, tmp_path):
    """-controller bdf: the BDF controller's trajectory, bit for bit its CPU
    restatement at the same tolerances, in the reference's output files."""
    build.build()
    m = synth.shorten(synth.make_c4_instance(7), 2.0, 21)
    m.atol = None
    inp, out = tmp_path / "in", tmp_path / "out"
    write_folder(m, str(inp))
    r = subprocess.run([build.CLI, str(inp), str(out), "-engine", "fp64", "-controller", "bdf",
                        "-rtol", "1e-7",
                        "-atol", "1e-10", "-max-order", "4", "-dump-f64", "-stats"],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ref, rst, rc = O.solve_bdf(m, rtol=1e-7, atol=1e-10, max_order=4)
    assert rc == 0
    full = read_table(out / "output" / "Solution.f64")
    assert np.array_equal(full[:, 1:], ref)
    import json
    st = json.loads((out / "output" / "stats.json").read_text())
    assert st["controller"] == "bdf" and st["be_steps"] == rst["steps"]
    assert st["order_final"] <= 4


def test_cli_stochastic_rescales_output(gpu, tmp_path):
    build.build()
    m = synth.tiny_network("reversible")
    inp, out = tmp_path / "in", tmp_path / "out"
    vol = 1e-18
    conv = vol * 6.022e23
    m_counts = synth.tiny_network("reversible")
    m_counts.x0 = m.x0 * conv
    m_counts.k = m.k.copy()
    m_counts.k[0] = m.k[0] / conv  # bimolecular: k * V * N_A in deterministic units
    write_folder(m_counts, str(inp))
    (inp / "modelkind").write_text("stochastic\n")
    (inp / "volume").write_text("%r\n" % vol)
    r = subprocess.run([build.CLI, str(inp), str(out), "-engine", "fp64", "-root", "sqrt",
                        "-dump-f64"],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    full = read_table(out / "output" / "Solution.f64")
    ref, _, _ = O.solve(m)
    assert np.allclose(full[:, 1:] / conv, ref, rtol=1e-9)
