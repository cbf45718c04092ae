"""Build the engine library and the CPU oracle in-tree.

libnqcd_gb300.so  (nqcdynamics.jl_gb300/nqcd_gb300/_lib/): the CUDA engine,
    sm_103a only.  The plain FP64 translation unit is compiled with
    -fmad=false so its arithmetic rounds exactly like the oracle's.
liboracle.so      (oracle/_build/): the FP64 CPU oracle, test
    infrastructure only (-ffp-contract=off for the same reason).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent.parent
CSRC = PKG_DIR.parent / "csrc"
LIB_DIR = PKG_DIR / "_lib"
BUILD_DIR = PKG_DIR.parent / "_build"
ORACLE_DIR = ROOT / "oracle"
ORACLE_BUILD = ORACLE_DIR / "_build"

ENGINE_LIB = LIB_DIR / "libnqcd_gb300.so"
ORACLE_LIB = ORACLE_BUILD / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# translation unit -> extra flags
ENGINE_UNITS = {
    "kernels_fp64.cu": ["-fmad=false"],
    "kernels_fp32.cu": [],
    "nqcd_abi.cu": [],
    "noalloc.cu": [],
    "mlp.cu": [],
    "kernels_iesh.cu": [],
    "tensor.cu": [],
    "kernels_tune.cu": [],
    "eigh.cu": [],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the engine cannot be built without the CUDA toolkit")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_engine(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "nqcd_gpu.h"]
    objs = []
    jobs = []
    for unit, flags in ENGINE_UNITS.items():
        src = CSRC / unit
        obj = BUILD_DIR / (unit + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                   *flags, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if force or _stale(ENGINE_LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(ENGINE_LIB), *map(str, objs), "-lcudart"])
    return ENGINE_LIB


def build_oracle(force: bool = False) -> Path:
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    srcs = sorted(ORACLE_DIR.glob("*.cpp"))
    deps = srcs + sorted(ORACLE_DIR.glob("*.h")) + sorted(CSRC.glob("*.h"))
    if force or _stale(ORACLE_LIB, deps):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
              *map(str, srcs), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_all(force: bool = False, verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_engine, force, verbose)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(force=True)
    print(ENGINE_LIB)
    print(ORACLE_LIB)
