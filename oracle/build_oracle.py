"""Build recipe of the oracle (test infrastructure only).

* oracle/liboracle_pbsm3d.so  <- oracle/pbsm3d_oracle.cpp (g++, OpenMP,
  -ffp-contract=off so x86 and Arm agree bit for bit);
* oracle/_ref/libref_atmosphere.so <- the reference's own
  src/physics/Atmosphere.cpp compiled where it lies in the reference tree
  (only when that tree is present), plus oracle/ref_atmosphere_shim.cpp.
  The rest of the reference PBSM3D path needs Boost, CGAL, Trilinos,
  MeteoIO and GSL, none of which exist here, so it is not built.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle_pbsm3d.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libref_atmosphere.so"
REFERENCE = Path(os.environ.get("CHM_REFERENCE", "/root/reference"))


def _cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_oracle(force: bool = False) -> Path:
    src = HERE / "pbsm3d_oracle.cpp"
    deps = [src, HERE / "pbsm3d_oracle.h", HERE.parent / "include" / "pbsm3d.h"]
    if force or not ORACLE_LIB.exists() or any(d.stat().st_mtime > ORACLE_LIB.stat().st_mtime for d in deps):
        _run([_cxx(), "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", str(src), "-o",
              str(ORACLE_LIB)])
    return ORACLE_LIB


def build_ref(force: bool = False) -> Path | None:
    atm = REFERENCE / "src" / "physics" / "Atmosphere.cpp"
    if not atm.exists():
        return REF_LIB if REF_LIB.exists() else None
    REF_DIR.mkdir(exist_ok=True)
    if force or not REF_LIB.exists():
        _run([_cxx(), "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", f"-I{REFERENCE / 'src'}",
              str(atm), str(HERE / "ref_atmosphere_shim.cpp"), "-o", str(REF_LIB)])
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
