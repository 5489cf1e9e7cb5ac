"""Builds libvlm_gb300.so in-tree (volcanor_gb300/_build/) for sm_103a.

FP64 translation units (bs64.cu, solver.cu, incr.cu) are compiled with -fmad=false and
the host units with -ffp-contract=off so that every FP64 operation rounds as
in the reference arithmetic; the FP32 kernel unit (bs32.cu) keeps FMA
contraction and flushes FP32 denormals (-ftz=true), which lets rsqrtf map to
a single MUFU instruction.  Compilation runs in parallel and takes well under a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libvlm_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_EXACT = ["bs64.cu", "solver.cu", "incr.cu"]
CU_FAST = ["bs32.cu"]
CU_PLAIN = ["noalloc.cu", "mlp.cu", "mlp_tc.cu", "surrogate.cu", "peak.cu"]
CXX = ["wing.cpp", "case.cpp", "plan.cpp"]


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def sources():
    return [SRC / f for f in CU_EXACT + CU_FAST + CU_PLAIN + CXX] + list(SRC.glob("*.h")) + [PKG.parent / "include" / "vlm.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc") if (cuda / "bin" / "nvcc").exists() else "nvcc"
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH]
    jobs = []
    objs = []
    for f in CU_EXACT:
        o = BUILD / (f + ".o")
        jobs.append([nvcc, *common, "-fmad=false", "-c", str(SRC / f), "-o", str(o)])
        objs.append(o)
    for f in CU_FAST:
        o = BUILD / (f + ".o")
        jobs.append([nvcc, *common, "-ftz=true", "-prec-div=false", "-prec-sqrt=false", "-c", str(SRC / f), "-o",
                     str(o)])
        objs.append(o)
    for f in CU_PLAIN:
        o = BUILD / (f + ".o")
        jobs.append([nvcc, *common, "-c", str(SRC / f), "-o", str(o)])
        objs.append(o)
    for f in CXX:
        o = BUILD / (f + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", f"-I{cuda / 'include'}", "-c",
                     str(SRC / f), "-o", str(o)])
        objs.append(o)
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    failed = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            print(" ".join(j))
            print(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(j[-3])
    if failed:
        raise RuntimeError(f"compilation failed: {failed}")
    tmp = BUILD / f"libvlm_gb300.{os.getpid()}.so"
    subprocess.check_call([nvcc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
    print(LIB)
