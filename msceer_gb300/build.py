"""Builds the native parts in-tree for sm_103a.

* ``msceer_gb300/libmsc_gpu.so``  -- the CUDA kernels + C ABI (include/msc_gpu.h)
* ``msceer_gb300/bin/steepest_lstar``, ``ondemandaccurate`` -- the drop-in CLIs (C++ over the C ABI)

Translation units compile in parallel with one ``-gencode`` so a fresh machine
builds in well under a minute.  ``python -m msceer_gb300.build`` runs it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmsc_gpu.so"
BIN = PKG / "bin"

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]
CU_SOURCES = ["lstar_kernels.cu", "ldir_kernels.cu", "grad_kernels.cu", "label_kernels.cu", "integrate_kernels.cu",
              "msc_capi.cu", "msc_labels_capi.cu", "conform_kernels.cu", "msc_static_scratch.cu", "triage_kernels.cu", "triage_prep.cu",
              "msc_triage_capi.cu", "ms_graph.cu", "saddle_lines.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmsc_gpu.so")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(map(str, cmd))}\n"
                           f"{res.stdout}\n{res.stderr}")
    return res


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append([nvcc, *GENCODE, *NVCC_FLAGS, "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *GENCODE, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"], verbose)
        os.replace(tmp, LIB)
    return LIB


def build_cli(verbose: bool = False, force: bool = False) -> Path:
    """The drop-in command lines (C++ over the C ABI): steepest_lstar, ondemandaccurate."""
    BIN.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    cuda = Path(_nvcc()).resolve().parent.parent
    cuda_lib = cuda / "lib64"
    for name in ("steepest_lstar", "ondemandaccurate"):
        exe = BIN / name
        src = PKG / "cli" / f"{name}.cpp"
        if force or _stale(exe, [src, LIB, ROOT / "include" / "msc_gpu.h"]):
            _run([cxx, "-O2", "-std=c++17", "-I", ROOT / "include", "-I", cuda / "include", src, "-o", exe,
                  "-L", PKG, "-lmsc_gpu", f"-Wl,-rpath,$ORIGIN/..", "-L", cuda_lib, "-lcudart",
                  f"-Wl,-rpath,{cuda_lib}"], verbose)
    return BIN / "steepest_lstar"


def build_oracle(verbose: bool = False) -> None:
    """The C oracle (test-only checker), and the reference harness when the
    reference sources are present on this machine."""
    _run(["make", "-s", "-C", ROOT / "oracle"], verbose)
    ref_root = Path(os.environ.get("MSC_REF_ROOT", "/root/reference"))
    if (ref_root / "include" / "gi_fast_robins_noalloc.h").exists():
        _run(["make", "-s", "-C", ROOT / "oracle", "ref", f"REF_ROOT={ref_root}"], verbose)


def build_all(verbose: bool = False, force: bool = False) -> None:
    build_library(verbose, force)
    build_cli(verbose, force)
    build_oracle(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(f"built {LIB}")
