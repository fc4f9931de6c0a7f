"""Build the in-tree shared libraries.

* ``3deye_gb300/lib3deye_gb300.so`` -- the CUDA kernels and the C-ABI of
  ``include/tde_capi.h`` (sm_103a only), plus the C++ reference API of
  ``include/3deye/``.
* ``oracle/liboracle.so`` -- the CPU oracle (test infrastructure).
* ``oracle/_ref/*.so`` -- the reference kernels compiled as C, only when
  TDE_REFERENCE names a checkout of the reference (test infrastructure).

Translation units compile in parallel; each one is rebuilt only when a source
or header it may include is newer than its object.
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
OUT_DIR = PKG / "_build"
LIB = PKG / "lib3deye_gb300.so"
ORACLE = ROOT / "oracle"
ORACLE_LIB = ORACLE / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Kernels whose float arithmetic must equal the CPU oracle's operation by
# operation are compiled without FMA contraction.
NO_FMAD = {"k_raycast.cu", "k_integrate.cu", "k_icp.cu", "k_depth.cu", "k_render.cu", "k_synth.cu", "k_rgbd.cu"}
CUDA_UNITS = ["capi.cu", "k_raycast.cu", "k_integrate.cu", "k_icp.cu", "k_depth.cu", "k_slab.cu",
              "pipeline.cu", "k_synth.cu", "noalloc.cu", "k_refiner.cu", "refiner.cu", "k_render.cu",
              "k_rgbd.cu"]
CXX_UNITS = ["wrappers.cpp"]
ORACLE_SOURCES = ["oracle.c", "oracle_scene.c", "oracle_f64.c", "oracle_rgbd.c"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build 3deye_gb300")


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    OUT_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").rglob("*.h"))
    units = [u for u in CUDA_UNITS + CXX_UNITS if (CSRC / u).exists()]
    jobs = []
    objs = []
    for u in units:
        src = CSRC / u
        obj = OUT_DIR / (u + ".o")
        objs.append(obj)
        if not _stale(obj, [src, Path(__file__)] + headers):
            continue
        if u.endswith(".cpp"):
            # host-only C++ (the reference API layer): no CUDA headers
            cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                   "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
            continue
        cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
               "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(CSRC),
               "-c", str(src), "-o", str(obj)]
        if u in NO_FMAD:
            cmd.append("-fmad=false")
        jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if _stale(LIB, objs) or jobs:
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    srcs = [ORACLE / s for s in ORACLE_SOURCES if (ORACLE / s).exists()]
    deps = srcs + list(ORACLE.glob("*.h"))
    if _stale(ORACLE_LIB, deps):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
              "-I", str(ROOT / "include"), *map(str, srcs), "-o", str(ORACLE_LIB), "-lm"])
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def build_reference_kernels(verbose: bool = False) -> None:
    """The reference's kernels compiled as C, when TDE_REFERENCE names a
    checkout of the reference (test infrastructure; skipped otherwise)."""
    script = ORACLE / "build_ref.sh"
    ref = os.environ.get("TDE_REFERENCE")
    if not ref or not (Path(ref) / "GPU" / "opencl").is_dir():
        return
    r = subprocess.run(["bash", str(script), ref], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference kernel build failed:\n" + r.stdout)
    if verbose:
        print(r.stdout)


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_or = ex.submit(build_oracle, verbose)
        f_lib.result()
        f_or.result()
    build_reference_kernels(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
