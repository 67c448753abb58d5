"""Callers of the C ABI without Python in the process.

tests/cabi/cabi_scf.cpp, compiled here against include/gansu_gb300.h and the
in-tree library, runs water STO-3G from files through molecule -> engine ->
core Hamiltonian -> RHF SCF and the allocation-free DIIS; the C++ HF_main
(dft_gansu_gb300/programs/hf_main.cpp, built by build()) runs the reference's
HF_main command line.  Energies against the reference-integral golden energy
(1e-8 Eh) and the Python API's (1e-9 Eh)."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import build, geometry

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"


def _cuda_home():
    return build._cuda_home()


def _keyvals(text):
    return {k: v for k, v in (line.split(None, 1) for line in text.splitlines() if " " in line)}


def test_cpp_caller_of_the_c_abi(built_library, cuda, tmp_path):
    exe = tmp_path / "cabi_scf"
    cuda_home = _cuda_home()
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", f"-I{ROOT / 'include'}", f"-I{cuda_home / 'include'}",
                    str(ROOT / "tests" / "cabi" / "cabi_scf.cpp"), "-o", str(exe), f"-L{build.PKG}", "-lgansu_gb300",
                    f"-L{cuda_home / 'lib64'}", "-lcudart", f"-Wl,-rpath,{build.PKG}",
                    f"-Wl,-rpath,{cuda_home / 'lib64'}"], check=True)
    xyz = tmp_path / "water.xyz"
    geometry.write_xyz(xyz, geometry.water())
    p = subprocess.run([str(exe), str(xyz), gg.basis_path("sto-3g")], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    kv = _keyvals(p.stdout)
    g = np.load(GOLDEN / "water_sto-3g.npz")
    assert int(kv["num_basis"]) == 7 and int(kv["num_electrons"]) == 10
    assert abs(float(kv["overlap_00"]) - float(g["S"][0, 0])) < 1e-13
    assert int(kv["converged"]) == 1
    assert abs(float(kv["total_energy"]) - float(g["energy_total"])) < 1e-8
    # second error = half the first: the weights (-1, 2) cancel the error, F = -1 * 1 + 2 * 3
    assert abs(float(kv["diis_noalloc_00"]) - 5.0) < 1e-12


def _hf_main(args, cwd):
    p = subprocess.run([str(build.HF_MAIN), *args], capture_output=True, text=True, cwd=cwd, timeout=600)
    assert p.returncode == 0, p.stderr + p.stdout
    return p.stdout


def _total(text):
    return float(re.search(r"Total Energy:\s*(\S+)", text).group(1))


def test_cpp_hf_main_rhf_recipe_and_molden(built_library, cuda, tmp_path):
    xyz = tmp_path / "water.xyz"
    geometry.write_xyz(xyz, geometry.water())
    recipe = tmp_path / "rhf.txt"
    recipe.write_text("# RHF with DIIS\nmethod = RHF\nconvergence_method = DIIS\ndiis_size = 8\n"
                      "convergence_energy_threshold = 1e-10\neri_method = stored\n")
    out = _hf_main(["-x", str(xyz), "-g", "sto-3g", "-p", str(recipe)], tmp_path)
    g = np.load(GOLDEN / "water_sto-3g.npz")
    assert abs(_total(out) - float(g["energy_total"])) < 1e-8
    assert "[Charge analysis]" in out and "Method: Restricted Hartree-Fock (RHF)" in out
    molden = (tmp_path / "output.molden").read_text()
    assert "[MO]" in molden and "[GTO]" in molden and molden.count("Ene=") == 7
    # a command-line value wins over the recipe's
    out2 = _hf_main(["-x", str(xyz), "-g", "sto-3g", "-p", str(recipe), "--convergence_method", "damping",
                     "--maxiter", "300"], tmp_path)
    assert "Convergence algorithm: damping" in out2
    assert abs(_total(out2) - float(g["energy_total"])) < 1e-6


OH_RADICAL = [(8, 0.0, 0.0, 0.0), (1, 0.0, 0.0, 0.97 * geometry.ANGSTROM_TO_BOHR)]


@pytest.mark.parametrize("args,method", [
    (["-m", "uhf"], "uhf"),
    (["-m", "rohf", "-c", "1"], "rohf"),
    (["--eri_method", "ri", "-ag", "cc-pvdz-rifit"], "ri"),
    (["--initial_guess", "sad", "--eigensolver", "purification"], "sad"),
])
def test_cpp_hf_main_matches_python_api(built_library, cuda, tmp_path, args, method):
    # UHF on the OH radical (the water cation's UHF needs ~90 iterations from the core guess)
    atoms = OH_RADICAL if method == "uhf" else geometry.water()
    xyz = tmp_path / "water.xyz"
    geometry.write_xyz(xyz, atoms)
    gbs = "cc-pvdz" if method == "ri" else "6-31g"
    out = _hf_main(["-x", str(xyz), "-g", gbs, "--convergence_energy_threshold", "1e-10", *args], tmp_path)
    pm = gg.ParameterManager()
    pm.parse_command_line_args(["-x", str(xyz), "-g", gg.basis_path(gbs), "--convergence_energy_threshold", "1e-10",
                                *[gg.basis_path(a) if a == "cc-pvdz-rifit" else a for a in args]])
    hf = gg.HFBuilder.buildHF(pm)
    e = hf.solve()
    assert hf.result["converged"] == 1 and "Converged: yes" in out
    # the OH radical's UHF energy surface is flat: runs that differ only in the order of the
    # Fock build's atomic additions stop (|dE| < 1e-10) at energies up to ~5e-8 apart
    assert abs(_total(out) - e) < (1e-7 if method == "uhf" else 1e-9), (out, e)
