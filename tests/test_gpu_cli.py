"""The command line (python -m dft_gansu_gb300), run as the reference's HF_main
and GeometryOptimization programs are: parameters from short options, --key
value pairs and a recipe file, the report on stdout, output.molden in the
working directory.  Energies equal the Python API's on the same parameters
(1e-10 Eh); the optimised water energy is the RHF/STO-3G minimum (1e-4 Eh)."""
import os
import re
import subprocess
import sys
from pathlib import Path

import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from dft_gansu_gb300.__main__ import main

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _energy(text):
    return float(re.search(r"Total energy:\s*(\S+)", text).group(1))


def test_hf_main_rhf_with_recipe(built_library, cuda, tmp_path, monkeypatch, capsys):
    xyz = tmp_path / "water.xyz"
    geometry.write_xyz(xyz, geometry.water())
    recipe = tmp_path / "rhf.txt"
    recipe.write_text("# RHF with DIIS\nmethod = RHF\nconvergence_method = DIIS\ndiis_size = 8\n"
                      "convergence_energy_threshold = 1e-10\n")
    monkeypatch.chdir(tmp_path)
    assert main(["-x", str(xyz), "-g", "6-31g_st", "-p", str(recipe)]) == 0
    out = capsys.readouterr().out
    molden = (tmp_path / "output.molden").read_text()
    assert "[MO]" in molden and "[GTO]" in molden

    pm = gg.ParameterManager()
    pm.parse_command_line_args(["-x", str(xyz), "-g", gg.basis_path("6-31g_st"),
                                "--convergence_energy_threshold", "1e-10"])
    hf = gg.HFBuilder.buildHF(pm)
    assert abs(_energy(out) - hf.solve()) < 1e-10


def test_hf_main_uhf_subprocess_and_sad_cache(built_library, cuda, tmp_path):
    xyz = tmp_path / "oh.xyz"
    geometry.write_xyz(xyz, [a for a in geometry.water()[:2]])  # OH radical
    r = subprocess.run([sys.executable, "-m", "dft_gansu_gb300", "-x", str(xyz), "-g", "sto-3g", "-m", "UHF",
                        "--convergence_energy_threshold", "1e-10", "--export_sad_cache", "1"],
                       cwd=tmp_path, capture_output=True, text=True, env=dict(os.environ, PYTHONPATH=str(ROOT)),
                       timeout=600)
    assert r.returncode == 0, r.stderr
    assert _energy(r.stdout) < -74.0
    assert (tmp_path / "output.molden").exists() and (tmp_path / "temp_sad_cache.dat").exists()


def test_geometry_optimization_program(built_library, cuda, tmp_path, monkeypatch, capsys):
    xyz = tmp_path / "w.xyz"
    atoms = [(z, x * 1.08 + 0.02 * i, y * 0.95, w + 0.01 * i) for i, (z, x, y, w) in enumerate(geometry.water())]
    geometry.write_xyz(xyz, atoms)
    monkeypatch.chdir(tmp_path)
    assert main(["GeometryOptimization", "-x", str(xyz), "-g", "sto-3g"]) == 0
    out = capsys.readouterr().out
    assert "Geometry optimization is completed." in out
    e = float(re.search(r"Final energy:\s*(\S+)", out).group(1))
    assert abs(e - (-74.9659)) < 1e-4
