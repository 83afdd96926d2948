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
