"""Builds libgansu_gb300.so (sm_103a) in-tree, in parallel, without cmake.

Every CUDA translation unit is compiled with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3``; the direct
Fock kernel source (csrc/fock_inst.cu) is compiled once per quartet class so
the 21 classes compile concurrently.  Objects are rebuilt only when a source
or header is newer than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgansu_gb300.so"
HF_MAIN = PKG / "HF_main"  # the C++ program (git-ignored build output)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# quartet classes (la, lb, lc, ld) with la>=lb, lc>=ld, (la,lb) >= (lc,ld)
FOCK_CLASSES = [
    (0, 0, 0, 0), (1, 0, 0, 0), (1, 0, 1, 0), (1, 1, 0, 0), (1, 1, 1, 0), (1, 1, 1, 1),
    (2, 0, 0, 0), (2, 0, 1, 0), (2, 0, 1, 1), (2, 0, 2, 0), (2, 1, 0, 0), (2, 1, 1, 0),
    (2, 1, 1, 1), (2, 1, 2, 0), (2, 1, 2, 1), (2, 2, 0, 0), (2, 2, 1, 0), (2, 2, 1, 1),
    (2, 2, 2, 0), (2, 2, 2, 1), (2, 2, 2, 2),
]

# longest translation units first (the pool starts them in this order)
CUDA_SOURCES = ["grad_class_f64_l5.cu", "grad_class_f64_l6.cu", "grad_class_f32_l56.cu", "grad_class_f64.cu",
                "grad_class_f32.cu", "grad.cu", "ri_grad.cu", "ri.cu", "batch.cu", "scf.cu", "engine.cu", "fock.cu",
                "fock_generic.cu", "one_electron.cu", "peaks.cu", "diis_noalloc.cu", "tc_gemm.cu", "purify.cu"]
CXX_SOURCES = ["molecule.cpp", "errors.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgansu_gb300")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + [ROOT / "include" / "gansu_gb300.h"]


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _jobs() -> list[tuple[list[str], Path, list[Path]]]:
    nvcc = _nvcc()
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    common = [nvcc, "-std=c++17", "-O3", "-lineinfo", ARCH, "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", *inc]
    hdr = _headers()
    jobs = []
    # the RI derivative kernels, one unit per auxiliary angular momentum (long units first)
    for lp in (3, 2, 1, 0):
        obj = BUILD / f"ri_grad_l{lp}.o"
        jobs.append(([*common, f"-DGB_RI_LP={lp}", "-c", str(CSRC / "ri_grad_inst.cu"), "-o", str(obj)], obj,
                     [CSRC / "ri_grad_inst.cu", *hdr]))
    for src in CUDA_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        jobs.append(([*common, "-c", str(CSRC / src), "-o", str(obj)], obj, [CSRC / src, *hdr]))
    for (a, b, c, d) in FOCK_CLASSES:
        obj = BUILD / f"fock_{a}{b}{c}{d}.o"
        defs = [f"-DGB_LA={a}", f"-DGB_LB={b}", f"-DGB_LC={c}", f"-DGB_LD={d}"]
        jobs.append(([*common, *defs, "-c", str(CSRC / "fock_inst.cu"), "-o", str(obj)], obj,
                     [CSRC / "fock_inst.cu", *hdr]))
    for src in CXX_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", *inc, "-c", str(CSRC / src), "-o", str(obj)]
        jobs.append((cmd, obj, [CSRC / src, *hdr]))
    return jobs


def _run(cmd: list[str]) -> tuple[int, str]:
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return p.returncode, p.stdout


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile (incrementally) and link the library; returns its path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    work = [(cmd, obj) for cmd, obj, deps in _jobs() if _stale(obj, deps)]
    objs = [obj for _, obj, _ in _jobs()]
    if work:
        n = jobs or max(1, min(len(work), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            futs = {ex.submit(_run, cmd): (cmd, obj) for cmd, obj in work}
            for fut in cf.as_completed(futs):
                rc, out = fut.result()
                cmd, obj = futs[fut]
                if rc != 0:
                    raise RuntimeError(f"compile failed for {obj.name}:\n{' '.join(cmd)}\n{out}")
                if verbose:
                    print(f"[build] {obj.name}", flush=True)
    if work or not LIB.exists() or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), "-shared", ARCH, "-o", str(tmp), *map(str, objs), "-lcublas", "-lcusolver"]
        rc, out = _run(cmd)
        if rc != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{out}")
        os.replace(tmp, LIB)
    build_programs()
    return LIB


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def build_programs() -> Path:
    """The C++ HF_main (programs/hf_main.cpp) over the C ABI, linked to the library."""
    src = PKG / "programs" / "hf_main.cpp"
    if _stale(HF_MAIN, [src, LIB, ROOT / "include" / "gansu_gb300.h"]):
        cuda = _cuda_home()
        tmp = HF_MAIN.with_suffix(".tmp")
        cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}", str(src), "-o", str(tmp),
               f"-L{PKG}", "-lgansu_gb300", f"-L{cuda / 'lib64'}", "-lcudart", "-Wl,-rpath,$ORIGIN",
               f"-Wl,-rpath,{cuda / 'lib64'}"]
        rc, out = _run(cmd)
        if rc != 0:
            raise RuntimeError(f"HF_main build failed:\n{' '.join(cmd)}\n{out}")
        os.replace(tmp, HF_MAIN)
    return HF_MAIN


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
