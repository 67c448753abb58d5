"""Command line of the engine, with the behaviour of the reference's two programs.

    python -m dft_gansu_gb300 -x water.xyz -g sto-3g -m rhf [--key value ...]

is HF_main (src/HF_main.cu:40-62): the parameters are parsed as
gansu::ParameterManager parses them (short options -m -v -p -x -g -ag -c,
``--key value`` pairs, a ``-p`` recipe file such as parameter_recipe/RHF_DIIS.txt
filling the keys not given), HFBuilder::buildHF makes the RHF, UHF or ROHF
object, which is solved, reported and written to output.molden in the working
directory; with export_sad_cache set, the SAD cache goes to temp_sad_cache.dat.
(The reference's HF_main tests that the key exists, which its defaults make
always true; here its value decides.)

    python -m dft_gansu_gb300 GeometryOptimization -x water.xyz -g sto-3g

is the GeometryOptimization program (src/GeometryOptimization.cu:37-47):
HFBuilder::buildOtimizer, then the final energy.

A basis given by name (``-g cc-pvdz``) is looked up among the bundled basis
files when no file of that name exists.  Errors of the engine (no GPU, an
invalid input) end the program with status 1 and the engine's message.
"""
from __future__ import annotations

import sys

from . import HFBuilder, HFError, ParameterManager, basis_path

PROGRAMS = ("HF_main", "GeometryOptimization")


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    program = "HF_main"
    if argv and argv[0] in PROGRAMS:
        program = argv.pop(0)
    params = ParameterManager()
    try:
        params.parse_command_line_args(argv)
    except KeyError as exc:
        print(f"error: {exc.args[0]}", file=sys.stderr)
        return 2
    if not params["xyzfilename"] or not params["gbsfilename"]:
        print("error: an xyz file (-x) and a basis set (-g) are required", file=sys.stderr)
        return 2
    try:
        params["gbsfilename"] = basis_path(params["gbsfilename"])
        if params["auxiliary_gbsfilename"]:
            params["auxiliary_gbsfilename"] = basis_path(params["auxiliary_gbsfilename"])
        if program == "GeometryOptimization":
            energy = HFBuilder.buildOtimizer(params)
            print("Geometry optimization is completed.")
            print(f"Final energy: {energy:.12f}")
            return 0
        hf = HFBuilder.buildHF(params)
        hf.solve()
        print(hf.report(), end="")
        hf.export_molden_file("output.molden")
        if params.get("export_sad_cache", bool):
            print("Exporting SAD cache to 'temp_sad_cache.dat'...")
            hf.export_sad_cache("temp_sad_cache.dat")
            print("SAD cache exported successfully.")
    except (HFError, FileNotFoundError, ValueError) as exc:
        print(f"error: {exc}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
