"""Host-side logic that needs no GPU: the C ABI library loads and exports every
declared symbol, the input model (basis/xyz parsing, primitive expansion,
CGTO factors) matches the oracle's independent restatement, the basis sizes of
the configured molecules, parameter handling and the geometry generators."""
import re
from pathlib import Path

import numpy as np
import pytest

import dft_gansu_gb300 as gg
from dft_gansu_gb300 import geometry
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "gansu_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^(?:int|void|long long|const char\s*\*)\s*(hf_[a-z0-9_]+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(built_library):
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(built_library, n), n
    from dft_gansu_gb300._capi import SIGNATURES
    assert set(SIGNATURES) == set(names)


def test_version_and_error_string(built_library):
    assert b"sm_103a" in built_library.hf_version()
    with pytest.raises(gg.HFError):
        gg.Molecular([(8, 0.0, 0.0, 0.0)], "/nonexistent.gbs")
    assert b"cannot open" in built_library.hf_last_error()


@pytest.mark.parametrize("atoms,gbs,nbf,nprim", [
    (geometry.water(), "sto-3g", 7, 15),
    (geometry.alkane(10), "6-31g_st", 194, 238),
    (geometry.alkane(10), "cc-pvdz", 260, 330),
    (geometry.c60(), "cc-pvdz", 900, 1320),
    (geometry.c60(), "cc-pvdz-rifit", 3960, 1080),
])
def test_basis_sizes(built_library, atoms, gbs, nbf, nprim):
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    assert mol.num_basis == nbf
    assert mol.num_primitives == nprim


@pytest.mark.parametrize("gbs", ["sto-3g", "6-31g_st", "cc-pvdz"])
def test_input_model_matches_oracle(built_library, gbs):
    atoms = geometry.alkane(3, seed=5)
    mol = gg.Molecular(atoms, gg.basis_path(gbs))
    b = O.make_basis(atoms, gg.basis_path(gbs))
    assert mol.num_basis == b.nbf
    np.testing.assert_allclose(mol.get_cgto_normalization_factors(), b.cgto, rtol=1e-14)
    t = mol.primitive_table()
    ref = b.reference_primitives()
    assert [r[0] for r in ref] == list(t["shell_type"])
    np.testing.assert_array_equal([r[4] for r in ref], t["basis_index"])
    np.testing.assert_allclose([r[1] for r in ref], t["exponent"])
    np.testing.assert_allclose([r[2] for r in ref], t["coefficient"])
    assert mol.num_electrons == sum(a[0] for a in atoms)


def test_cgto_quirk_for_p_functions(built_library):
    # the reference normalisation leaves contracted p functions non-unit (L/2 integer division)
    mol = gg.Molecular(geometry.water(), gg.basis_path("sto-3g"))
    f = mol.get_cgto_normalization_factors()
    b = O.make_basis(geometry.water(), gg.basis_path("sto-3g"))
    S, _, _ = O.one_electron(b)
    assert abs(S[2, 2] - 1.0) > 0.1  # O 2px
    assert abs(S[0, 0] - 1.0) < 1e-8  # O 1s
    assert np.all(f > 0)


def test_xyz_parser_matches_oracle(built_library, tmp_path):
    p = tmp_path / "dec.xyz"
    geometry.write_xyz(p, geometry.alkane(10))
    mol = gg.Molecular.from_files(p, gg.basis_path("6-31g_st"))
    ref = O.parse_xyz(p)
    got = mol.get_atoms()
    assert len(got) == len(ref) == 32
    for a, r in zip(got, ref):
        assert a[0] == r[0]
        np.testing.assert_allclose(a[1:], r[1:], atol=1e-9)


def test_xyz_rejects_overlapping_atoms(built_library, tmp_path):
    p = tmp_path / "bad.xyz"
    p.write_text("2\nbad\nH 0 0 0\nH 0 0 0.00001\n")
    with pytest.raises(gg.HFError):
        gg.Molecular.from_files(p, gg.basis_path("sto-3g"))


def test_odd_electron_count_reported(built_library):
    mol = gg.Molecular([(1, 0.0, 0.0, 0.0)], gg.basis_path("sto-3g"))
    assert (mol.num_alpha_spins, mol.num_beta_spins) == (1, 0)


def test_parameter_manager_rules(tmp_path):
    pm = gg.ParameterManager()
    assert pm["eri_method"] == "stored" and pm.get("diis_size", int) == 8
    pm["method"] = "RHF"
    assert pm["method"] == "rhf"
    pm["gbsfilename"] = "Basis/STO-3G.gbs"
    assert pm["gbsfilename"] == "Basis/STO-3G.gbs"
    with pytest.raises(KeyError):
        pm["not_a_key"] = 1
    rec = tmp_path / "r.txt"
    rec.write_text("convergence_method = DIIS\ndiis_size = 6\n# comment\n")
    pm.load_from_file(rec)
    assert pm.get("diis_size", int) == 6 and pm["convergence_method"] == "diis"


def test_reference_recipes_parse():
    """Every recipe of the reference's parameter_recipe/ (RHF, UHF, ROHF with DIIS,
    damping and optimal damping, the evaluation recipe) loads into the mirror with
    the reference's values, so HF_main recipes run unchanged."""
    from oracle import oracle as O
    if O.REFERENCE_ROOT is None:
        pytest.skip("GANSU_REFERENCE not set")
    recipes = sorted((O.REFERENCE_ROOT / "parameter_recipe").glob("*.txt"))
    if not recipes:
        pytest.skip("reference tree not mounted")
    for f in recipes:
        pm = gg.ParameterManager()
        pm.load_from_file(f)
        assert pm["method"] == f.name.split("_")[0].lower()
        assert pm["convergence_method"] in ("diis", "damping", "optimaldamping")
        assert pm.get("diis_include_transform", bool) is False
        assert 0.0 < pm.get("damping_factor", float) <= 1.0
        assert 0.0 < pm.get("convergence_energy_threshold", float) <= 1e-6
    ev = gg.ParameterManager()
    ev.load_from_file(O.REFERENCE_ROOT / "parameter_recipe" / "RHF_eval.txt")
    assert ev["initial_guess"] == "sad" and ev.get("schwarz_screening_threshold", float) == 1e-13


def test_geometries():
    dec = geometry.alkane(10, jitter=0.0)
    x = np.array([a[1:] for a in dec]) / geometry.ANGSTROM_TO_BOHR
    cc = np.linalg.norm(x[0] - x[1])
    assert abs(cc - 1.54) < 1e-9
    hs = [np.linalg.norm(x[i] - x[j]) for i in range(10) for j in range(10, 32) if np.linalg.norm(x[i] - x[j]) < 1.2]
    assert len(hs) == 22 and np.allclose(hs, 1.09)
    ch4 = np.array([a[1:] for a in geometry.alkane(1, jitter=0.0)]) / geometry.ANGSTROM_TO_BOHR
    assert [a[0] for a in geometry.alkane(1)] == [6, 1, 1, 1, 1]
    assert np.allclose(np.linalg.norm(ch4[1:] - ch4[0], axis=1), 1.09)
    c = np.array([a[1:] for a in geometry.c60(jitter=0.0)]) / geometry.ANGSTROM_TO_BOHR
    d = np.linalg.norm(c[:, None] - c[None], axis=-1)
    bonds = np.sort(d[(d > 0.1) & (d < 1.6)])
    assert len(bonds) == 180 and set(np.round(bonds, 6)) == {1.4, 1.45}
    clusters = geometry.water_cluster_set(16, seed=2)
    for cl in clusters:
        o = np.array([a[1:] for a in cl if a[0] == 8]) / geometry.ANGSTROM_TO_BOHR
        if len(o) > 1:
            dd = np.linalg.norm(o[:, None] - o[None], axis=-1) + np.eye(len(o)) * 9
            assert dd.min() >= 2.7 - 1e-9


def test_sad_format_roundtrip_and_atom_ranges(built_library, tmp_path):
    """.sad write/read round trip (read_density_from_sad format) and the atoms'
    basis ranges against the oracle's."""
    from dft_gansu_gb300 import sad
    from oracle import oracle as O

    rng = np.random.default_rng(0)
    dens = {"H": (rng.normal(size=(2, 2)), rng.normal(size=(2, 2))),
            "O": (rng.normal(size=(9, 9)), rng.normal(size=(9, 9)))}
    sad.write_sad(tmp_path / "x.sad", dens)
    back = sad.read_sad(tmp_path / "x.sad")
    for el in dens:
        for i in range(2):
            np.testing.assert_allclose(back[el][i], dens[el][i], rtol=1e-10)
    atoms = geometry.alkane(3, jitter=0.02, seed=1)
    for gbs in ("6-31g", "cc-pvdz"):
        mol = gg.Molecular(atoms, gg.basis_path(gbs))
        assert sad.atom_basis_ranges(mol) == O.atom_ranges(O.make_basis(atoms, gg.basis_path(gbs)))
    sad.export_sad_cache(tmp_path / "c.dat", dens["O"][0], dens["O"][1])
    toks = (tmp_path / "c.dat").read_text().split()
    assert toks[0] == "9" and len(toks) == 1 + 2 * 81


def test_pure_function_counts(built_library):
    """Pure (spherical) function counts of the benchmark inputs: the spherical sizes
    quoted for them (decane cc-pVDZ 250, C60 cc-pVDZ 840, cc-pVDZ-RIFIT 3360 needs f
    shells and is not built); the transform's d block spans the pure functions."""
    from dft_gansu_gb300 import spherical

    dec = gg.Molecular(geometry.alkane(10, jitter=0.02, seed=0), gg.basis_path("cc-pvdz"))
    assert dec.num_basis == 260 and spherical.num_pure(dec) == 250
    c60 = gg.Molecular(geometry.c60(), gg.basis_path("cc-pvdz"))
    assert c60.num_basis == 900 and spherical.num_pure(c60) == 840
    T = spherical.transform(dec)
    assert T.shape == (260, 250) and np.linalg.matrix_rank(T) == 250
    # the pure d combinations carry no r^2 = xx + yy + zz component (coefficient space)
    assert np.allclose(spherical.D_PURE.T @ np.array([1, 1, 1, 0, 0, 0.0]), 0.0)


def test_command_line_rejects_bad_arguments(capsys):
    """The HF_main front end stops on its arguments before any device work."""
    from dft_gansu_gb300.__main__ import main
    assert main(["--no_such_key", "1"]) == 2
    assert "no_such_key" in capsys.readouterr().err
    assert main(["-m", "rhf"]) == 2  # no xyz file, no basis
    assert "required" in capsys.readouterr().err
    assert main(["-x"]) == 2  # option without a value


def test_public_header_compiles_as_c():
    """include/gansu_gb300.h is a C header: tests/cabi/header_c_check.c takes the
    address of entry points with their declared types (gcc, -Werror)."""
    import shutil
    import subprocess
    root = Path(__file__).resolve().parents[1]
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", f"-I{root / 'include'}", "-fsyntax-only",
                    str(root / "tests" / "cabi" / "header_c_check.c")], check=True)


def test_reference_side_plugin_compiles_against_reference_headers(tmp_path):
    """The gansu::ERI plugins and gansu::gpu shims (dft_gansu_gb300/plugin/) compile
    against the reference's own include/eri.hpp, rhf.hpp, uhf.hpp and gpu_manager.hpp."""
    import subprocess
    from oracle import oracle as O
    from dft_gansu_gb300 import build as b
    if O.REFERENCE_ROOT is None:
        pytest.skip("GANSU_REFERENCE not set")
    root = Path(__file__).resolve().parents[1]
    ref = O.REFERENCE_ROOT
    subprocess.run([b._nvcc(), "-std=c++17", f"-I{root / 'include'}", f"-I{ref / 'include'}", f"-I{ref / 'src'}",
                    f"-I{root / 'dft_gansu_gb300' / 'plugin'}", "-c",
                    str(root / "dft_gansu_gb300" / "plugin" / "plugin_check.cu"), "-o", str(tmp_path / "p.o")],
                   check=True)


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the header's structs (dft_gansu_gb300/_capi.py) have the
    C layout: sizeof and every field's offset from a C program built with gcc."""
    import ctypes
    import shutil
    import subprocess
    from dft_gansu_gb300 import _capi
    root = Path(__file__).resolve().parents[1]
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    structs = {"hf_primitive_shell": _capi.PrimitiveShell, "hf_atom": _capi.Atom,
               "hf_scf_options": _capi.ScfOptions, "hf_scf_result": _capi.ScfResult,
               "hf_autotune_report": _capi.AutotuneReport}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gansu_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{root / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
