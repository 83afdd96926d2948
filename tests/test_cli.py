"""CLI argument and input-folder errors exit with the reference's codes
(simulator.cu:61-280, Simulation.cuh:373-391); they occur before any GPU
work, so they are checked without a GPU."""
import os
import subprocess

import pytest

from lassie_gb300 import build, synth
from lassie_gb300.model import write_folder


@pytest.fixture(scope="module")
def cli():
    build.build()
    return build.CLI


def run(cli, *args):
    return subprocess.run([cli, *args], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                          text=True, timeout=60).returncode


def code(c):
    return c & 0xff


def test_no_arguments(cli):
    assert run(cli) == code(-3)


def test_missing_output(cli, tmp_path):
    assert run(cli, str(tmp_path)) == code(-2)


def test_missing_input_folder(cli, tmp_path):
    assert run(cli, str(tmp_path / "nope"), str(tmp_path / "out")) == code(-1)


def test_missing_mandatory_files(cli, tmp_path):
    inp = tmp_path / "in"
    inp.mkdir()
    assert run(cli, str(inp), str(tmp_path / "out")) == code(-4)


def test_bad_precision_flag(cli, tmp_path):
    inp = tmp_path / "in"
    write_folder(synth.tiny_network("decay"), str(inp))
    assert run(cli, str(inp), str(tmp_path / "out"), "-p") == code(-5)
    assert run(cli, str(inp), str(tmp_path / "out"), "-p", "half") == code(-6)


def test_bad_modelkind_and_volume(cli, tmp_path):
    inp = tmp_path / "in"
    write_folder(synth.tiny_network("decay"), str(inp))
    (inp / "modelkind").write_text("banana\n")
    assert run(cli, str(inp), str(tmp_path / "o1")) == code(-7)
    (inp / "modelkind").write_text("stochastic\n")
    assert run(cli, str(inp), str(tmp_path / "o2")) == code(-8)
    (inp / "volume").write_text("1e-15\n")
    (inp / "left_side").write_text("1\t1\t1\n")
    (inp / "right_side").write_text("0\t0\t0\n")
    (inp / "M_0").write_text("1\t1\t1\n")
    assert run(cli, str(inp), str(tmp_path / "o3")) == code(-12)


def test_output_folder_created(cli, tmp_path):
    inp = tmp_path / "in"
    write_folder(synth.tiny_network("decay"), str(inp))
    (inp / "modelkind").write_text("banana\n")
    run(cli, str(inp), str(tmp_path / "newout"))
    assert os.path.isdir(tmp_path / "newout" / "output")


def test_symbolic_odes_and_jacobian(cli, tmp_path):
    """-v2/-v3 print the ODE system and the Jacobian before integrating,
    in the reference's notation (Simulation.cuh:83-228): A + B -> 2C,
    2C -> A, 0 -> B; species 1 fed in a second run (its ODE line is
    omitted and its Jacobian column is 0)."""
    import numpy as np
    from lassie_gb300.model import Model
    m = Model(left=np.array([[1, 1, 0], [0, 0, 2], [0, 0, 0]]),
              right=np.array([[0, 0, 2], [1, 0, 0], [0, 1, 0]]),
              k=np.array([0.5, 0.2, 0.1]), x0=np.array([1.0, 1.0, 0.0]), t=np.linspace(0, 1, 3))
    write_folder(m, str(tmp_path / "in"))
    r = subprocess.run([cli, str(tmp_path / "in"), str(tmp_path / "out"), "-v3"],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    lines = r.stdout.splitlines()
    odes = [ln for ln in lines if ln.startswith("dx[") and "][" not in ln]
    jac = [ln for ln in lines if ln.startswith("dx[") and "][" in ln]
    assert odes == ["dx[0] = -1*k[0]*x[0]*x[1]+1*k[1]*x[2]*x[2]",
                    "dx[1] = -1*k[0]*x[0]*x[1]+1*k[2]",
                    "dx[2] = +2*k[0]*x[0]*x[1]-2*k[1]*x[2]*x[2]"]
    assert jac == ["dx[0][0] = -1*k[0]*x[1]", "dx[0][1] = -1*k[0]*x[0]", "dx[0][2] = 2*k[1]*x[2]",
                   "dx[1][0] = -1*k[0]*x[1]", "dx[1][1] = -1*k[0]*x[0]", "dx[1][2] = 0",
                   "dx[2][0] = +2*k[0]*x[1]", "dx[2][1] = +2*k[0]*x[0]", "dx[2][2] = -4*k[1]*x[2]"]
    m.feed = np.array([0.0, 1.0, 0.0])
    write_folder(m, str(tmp_path / "fed"))
    r = subprocess.run([cli, str(tmp_path / "fed"), str(tmp_path / "out2"), "-v3"],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    lines = r.stdout.splitlines()
    assert not any(ln.startswith("dx[1] =") for ln in lines)
    assert "dx[0][1] = 0" in lines and "dx[2][1] = 0" in lines
