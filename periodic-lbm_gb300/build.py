"""Build libplbmgpu.so in-tree from csrc/ with nvcc for sm_103a.

Each translation unit is compiled separately (in parallel) and the objects are
linked into one shared library next to this file.  step_f64.cu is compiled
twice: with FMA contraction (namespace plbm::fma) and without it
(-DPLBM_STRICT --fmad=false, namespace plbm::strict).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
BUILD = HERE / "_build"
LIB = HERE / "libplbmgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}"]

# (source, object, extra flags)
UNITS = [
    ("step_f64.cu", "step_f64_fma.o", ["--fmad=true"]),
    ("step_f64.cu", "step_f64_strict.o", ["--fmad=false", "-DPLBM_STRICT"]),
    ("step_dev.cu", "step_dev.o", ["--fmad=true"]),
    ("step_df64.cu", "step_df64.o", ["--fmad=false"]),
    ("fields.cu", "fields.o", ["--fmad=false"]),
    ("noalloc.cu", "noalloc.o", ["--fmad=false"]),
    ("batched.cu", "batched.o", ["--fmad=true"]),
    ("adjoint.cu", "adjoint.o", ["--fmad=true"]),
    ("grid.cpp", "grid.o", ["-x", "cu", "--fmad=false"]),
    ("grid_io.cpp", "grid_io.o", ["-x", "cu", "--fmad=false"]),
    ("plugin.cpp", "plugin.o", ["-x", "cu", "--fmad=false"]),
    ("batch.cpp", "batch.o", ["-x", "cu", "--fmad=false"]),
    ("adjoint.cpp", "adjoint_host.o", ["-x", "cu", "--fmad=false"]),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libplbmgpu.so")


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile csrc/ into libplbmgpu.so; returns the library path."""
    cc = nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    jobs = []
    for src, obj, extra in UNITS:
        srcp = CSRC / src
        if not srcp.exists():
            continue
        objp = BUILD / obj
        if force or _stale(objp, [srcp, *headers, Path(__file__)]):
            cmd = [cc, *ARCH, *COMMON, *extra, "-c", str(srcp), "-o", str(objp)]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd))
            if r.stderr:
                print(r.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    objs = [str(BUILD / obj) for src, obj, _ in UNITS if (CSRC / src).exists()]
    if force or jobs or not LIB.exists() or _stale(LIB, [Path(o) for o in objs]):
        cmd = [cc, *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
