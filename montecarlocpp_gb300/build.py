"""Build the in-tree C-ABI library libmc_gb300.so for sm_103a with nvcc.

Three translation units compiled in parallel (FP32 kernels, FP64 kernels
with --fmad=false, host API), linked into montecarlocpp_gb300/_build/.
No cmake, no torch extension machinery: the library links only cudart.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmc_gb300.so")
MAIN = os.path.join(OUT, "mc_main")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]
UNITS = {
    "mc_f32.cu": [],
    "mc_f64.cu": ["--fmad=false"],
    "mc_api.cu": [],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the GB300 kernels cannot be built")


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "mc_gb300.h"), os.path.join(HERE, "..", "include", "mc_gb300.hpp")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    if not os.path.exists(MAIN):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources() if os.path.exists(s))


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()

    def one(item):
        src, extra = item
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *extra, *os.environ.get("MC_NVCC_FLAGS", "").split(), "-c",
               os.path.join(CSRC, src), "-o", obj]
        if ptxas_v:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose or ptxas_v:
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(one, UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # C++ driver over the C++ mirror of the reference API
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", os.path.join(CSRC, "mc_main.cpp"), "-I", os.path.join(HERE, "..", "include"),
           "-L", OUT, "-lmc_gb300", "-Wl,-rpath,$ORIGIN", "-o", MAIN]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"mc_main build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="-v" in sys.argv)
    print(LIB)
