"""Builds the native parts of amcl3d_gb300 in-tree.

* ``_lib/libamcl3d_gpu.so``: the CUDA kernels and the C ABI declared in
  ``include/amcl3d_gpu.h``, compiled for sm_103a only;
* ``_lib/libamcl3d_dropin.so``: the C++ ``amcl3d::Grid3d`` / ``amcl3d::ParticleFilter``
  classes over the C ABI, built against the test stand-in headers (a ROS build
  compiles ``cpp/*.cpp`` against the real ones instead).

Every translation unit compiles in parallel; objects are cached by source
timestamps under ``_build/``.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
CPP = PKG / "cpp"
BUILD = PKG / "_build"
LIB = PKG / "_lib"
INCLUDE = ROOT / "include"
# Stand-in ROS/PCL/octomap/boost headers (types only) for builds without ROS installed.
SHIM = ROOT / "tests" / "stand_in"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    # Reproducing the reference's rounding needs a*b+c kept as two roundings
    # everywhere (device and host): no FMA contraction.
    "--fmad=false",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off",
    "-Xptxas",
    "-warn-spills",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build amcl3d_gb300")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_gpu(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + [INCLUDE / "amcl3d_gpu.h"]
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))  # .cpp: host-only units
    objs = []
    jobs = []
    nv = nvcc()
    for src in sources:
        obj = BUILD / (src.name.replace(".", "_") + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nv, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    so = LIB / "libamcl3d_gpu.so"
    if force or jobs or _stale(so, objs):
        _run([nv, *ARCH, "-shared", "-o", str(so), *map(str, objs), "-lcudart"])
    return so


def build_dropin(force: bool = False) -> Path:
    """C++ drop-in classes (namespace amcl3d) linked against libamcl3d_gpu.so."""
    LIB.mkdir(exist_ok=True)
    so = LIB / "libamcl3d_dropin.so"
    srcs = sorted(CPP.glob("*.cpp"))
    hdrs = sorted(CPP.glob("*.h")) + [INCLUDE / "amcl3d_gpu.h"]
    if not srcs:
        return so
    if force or _stale(so, srcs + hdrs + [LIB / "libamcl3d_gpu.so"]):
        cxx = os.environ.get("CXX", "g++")
        _run([
            cxx, "-std=c++14", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
            f"-I{CPP}", f"-I{INCLUDE}", f"-I{SHIM}",
            "-o", str(so), *map(str, srcs),
            f"-L{LIB}", "-lamcl3d_gpu", f"-Wl,-rpath,{LIB}",
        ])
    return so


def build_oracle() -> None:
    """The C restatement (always) and, where the reference tree exists, the
    reference filter core compiled verbatim (test infrastructure only)."""
    mk = ROOT / "oracle" / "Makefile"
    _run(["make", "-s", "-C", str(mk.parent), "all"])
    # the reference checkout: AMCL3D_REF_ROOT, else a `reference` directory beside this one
    ref_root = Path(os.environ.get("AMCL3D_REF_ROOT", str(ROOT.parent / "reference")))
    ref = Path(os.environ.get("AMCL3D_REF_SRC", str(ref_root / "amcl3d" / "src")))
    if (ref / "ParticleFilter.cpp").exists():
        _run(["make", "-s", "-C", str(mk.parent), "ref", f"REF_SRC={ref}"])


def build_all(force: bool = False) -> None:
    build_gpu(force)
    build_dropin(force)
    build_oracle()


if __name__ == "__main__":
    import sys

    build_all(force="--force" in sys.argv)
    print("built", LIB)
