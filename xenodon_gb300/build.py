"""Build the native parts of xenodon_gb300 in-tree.

    python -m xenodon_gb300.build            # library + CLI
    python -m xenodon_gb300.build --clean

Produces
    xenodon_gb300/lib/libxenodon.so   the C-ABI library (include/xenodon.h):
                                      CUDA kernels for sm_103a + host code
    xenodon_gb300/bin/xenodon         the `xenodon render|convert` CLI

CUDA sources are compiled with nvcc for sm_103a only, with --fmad=false so
that the traversal kernels round like the reference shaders (explicit fmaf()
calls still fuse).  Host C++ is compiled with -ffp-contract=off for the same
reason: the Arm host compiler would otherwise fuse multiply-adds.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
OBJ = PKG / "_build"
LIB = PKG / "lib" / "libxenodon.so"
CLI = PKG / "bin" / "xenodon"
INCLUDE = ROOT / "include"

ARCH = os.environ.get("XN_CUDA_ARCH", "103a")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC)")


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


NVCC_FLAGS = [
    f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-Xptxas", "-warn-spills",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall", "-Wextra"]


def _deps(src: Path) -> list[Path]:
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    headers += list(HOST.glob("*.h"))
    return [src, *headers]


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        sys.stderr.write(p.stdout + p.stderr)
        raise RuntimeError("build failed: " + " ".join(cmd))


def _compile(src: Path) -> Path:
    out = OBJ / (src.stem + (".cu.o" if src.suffix == ".cu" else ".o"))
    if _stale(out, _deps(src)):
        if src.suffix == ".cu":
            _run([nvcc(), *NVCC_FLAGS, f"-I{INCLUDE}", "-c", str(src), "-o", str(out)])
        else:
            _run(["g++", *CXX_FLAGS, f"-I{INCLUDE}", f"-I{cuda_home() / 'include'}", "-c", str(src), "-o", str(out)])
    return out


def build(verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    lib_srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    cli_srcs = sorted(HOST.glob("*.cpp"))
    with ThreadPoolExecutor(max_workers=max(2, min(16, os.cpu_count() or 2))) as ex:
        lib_objs = list(ex.map(_compile, lib_srcs))
        cli_objs = list(ex.map(_compile, cli_srcs))
    if _stale(LIB, lib_objs):
        _run([nvcc(), f"-gencode=arch=compute_{ARCH},code=sm_{ARCH}", "-shared", "--cudart", "static",
              "-o", str(LIB), *map(str, lib_objs), "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"])
    if cli_objs:
        CLI.parent.mkdir(exist_ok=True)
        if _stale(CLI, cli_objs + [LIB]):
            _run(["g++", "-o", str(CLI), *map(str, cli_objs), f"-L{LIB.parent}", "-lxenodon",
                  "-Wl,-rpath,$ORIGIN/../lib", "-lpthread"])
    if verbose:
        print(f"built {LIB}" + (f" and {CLI}" if cli_objs else ""))
    return LIB


def clean() -> None:
    for p in (OBJ, LIB.parent, CLI.parent):
        if p.exists():
            shutil.rmtree(p)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--clean", action="store_true")
    a = ap.parse_args(argv)
    if a.clean:
        clean()
    else:
        build(verbose=True)


if __name__ == "__main__":
    main()
