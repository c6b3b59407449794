"""The drop-in CLI shells (tl_cli, tl_gen)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tau_leaping_gb300 import Model

PKG = Path(__file__).resolve().parents[1] / "tau_leaping_gb300"


def run(args, cwd):
    return subprocess.run([str(PKG / args[0]), *args[1:]], capture_output=True, text=True, cwd=cwd, timeout=300)


def test_gen_writes_readable_models(tmp_path):
    r = run(["tl_gen", "-s", "-r", "20", "-o", str(tmp_path / "c.xml")], tmp_path)
    assert r.returncode == 0, r.stderr
    m = Model.from_stochkit(tmp_path / "c.xml")
    assert (m.n_species, m.n_channels) == (20, 200)
    assert run(["tl_gen", "-w", "-r", "16", "-o", str(tmp_path / "w.xml")], tmp_path).returncode == 0
    assert Model.from_stochkit(tmp_path / "w.xml").n_channels == 16
    assert run(["tl_gen", "--bogus"], tmp_path).returncode == 2


def test_cli_argument_errors(tmp_path):
    assert run(["tl_cli"], tmp_path).returncode == 2
    assert run(["tl_cli", "-f", "x.xml", "-t", "0", "-n", "4"], tmp_path).returncode == 2
    r = run(["tl_cli", "-f", str(tmp_path / "missing.xml"), "-t", "1", "-n", "4", "-r", "S1"], tmp_path)
    assert r.returncode == 1 and "I/O error" in r.stderr


@pytest.mark.gpu
def test_cli_writes_reference_format(tmp_path):
    m = Model.generate("dimer", x0_min=2000, x0_max=2000)
    xml = tmp_path / "d.xml"
    m.write_stochkit(xml)
    r = run(["tl_cli", "-f", str(xml), "-t", "1", "-n", "500", "-r", "S1", "S2", "-i", "4", "-b", "run",
             "--seed", "3"], tmp_path)
    assert r.returncode == 0, r.stderr
    assert "It took" in r.stdout
    mean = np.loadtxt(tmp_path / "mean_run.txt")
    sd = np.loadtxt(tmp_path / "stddev_run.txt")
    assert mean.shape == (5, 3) and sd.shape == (5, 3)
    ref = Model.from_stochkit(xml).simulate(1.0, 500, seed=3, intervals=4, tracked=[0, 1])
    assert np.allclose(mean[:, 0], ref.times[0], rtol=1e-5)
    assert np.allclose(mean[:, 1:], ref.mean[0], rtol=1e-5)
    assert np.allclose(sd[:, 1:], ref.stddev[0], rtol=1e-5)
