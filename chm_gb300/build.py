"""Build libpbsm3d_cuda.so (sm_103a) in-tree with nvcc.

The CUDA sources are compiled in parallel, one object per translation unit,
then linked into chm_gb300/lib/libpbsm3d_cuda.so against the CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "chm_gb300" / "csrc"
LIBDIR = ROOT / "chm_gb300" / "lib"
BUILD = ROOT / "_build"
LIB = LIBDIR / "libpbsm3d_cuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr"]
# the mesh reader's geometry matches CHM's operation order on every host (no FMA contraction)
PER_FILE: dict = {"mesh_io.cu": ["-Xcompiler", "-ffp-contract=off"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpbsm3d_cuda")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    srcs = _sources()
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "pbsm3d.h"]
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    nv = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            cmd = [nv, *NVFLAGS, *ARCH, *PER_FILE.get(src.name, []), "-c", str(src), "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
            if verbose:
                print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or _stale(LIB, objs):
        cmd = [nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


SHIM = ROOT / "chm_gb300" / "shim"
HARNESS = LIBDIR / "pbsm3d_harness"


def build_shim(force: bool = False) -> Path:
    """The C++ module (CHM module_base replica + PBSM3D over the C ABI) and its
    harness executable, linked against libpbsm3d_cuda.so."""
    lib = build_cuda()
    srcs = [SHIM / "PBSM3D_gpu.cpp", SHIM / "harness.cpp"]
    deps = srcs + [SHIM / "PBSM3D_gpu.hpp", SHIM / "chm_module.hpp", ROOT / "include" / "pbsm3d.h", lib]
    if force or _stale(HARNESS, deps):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        cmd = [cxx, "-std=c++17", "-O2", *map(str, srcs), "-o", str(HARNESS), f"-L{LIBDIR}", "-lpbsm3d_cuda",
               f"-Wl,-rpath,{LIBDIR}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"shim build failed:\n{r.stdout}\n{r.stderr}")
    return HARNESS


if __name__ == "__main__":
    print(build_cuda(force=True, verbose=True))
