"""Build the tracker's shared library in-tree: ``libfrg_gb300.so`` next to this file.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked with the
host C++ translation unit into one C-ABI shared library (include/frg_gb300.h).
Runs with nvcc alone (no cmake, no torch); the same recipe builds on x86 and on
the aarch64 GPU hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfrg_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["frg_track.cu", "frg_track_team.cu", "frg_capi.cu", "frg_noalloc.cu", "frg_mlp.cu", "frg_dcoll.cu"]
# The tracking kernels' FP32 arithmetic is checked by residuals and finished in FP64,
# so FP32 division and square root use the fast approximate forms (a few ulp) and FP32
# subnormals flush to zero; FP64 arithmetic is unaffected by these flags.
SOURCE_FLAGS = {"frg_track.cu": ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
                "frg_track_team.cu": ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]}
STAMP = os.path.join(BUILD, "flags.txt")


def _extra_flags() -> list:
    """Additional nvcc flags for the CUDA sources from FRG_NVCC_FLAGS (space separated)."""
    return os.environ.get("FRG_NVCC_FLAGS", "").split()
CXX_SOURCES = ["frg_collect.cpp"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfrg_gb300.so")
    return path


def _sources_newer_than(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(HERE, "..", "include", "frg_gb300.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    """Compile (if stale) and return the path of libfrg_gb300.so."""
    flags_id = " ".join(_extra_flags())
    old_id = open(STAMP).read() if os.path.exists(STAMP) else ""
    if not force and not _sources_newer_than(LIB) and old_id == flags_id:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", CSRC, "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        cmd = [cc, *ARCH, *common, *SOURCE_FLAGS.get(src, []), *_extra_flags(), "-c", os.path.join(CSRC, src),
               "-o", obj]
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        jobs.append((cmd, obj))
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        cmd = [cc, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(HERE, "..", "include"),
               "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))

    def run(job):
        cmd, _ = job
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(run, jobs))
    if ptxas_info or verbose:
        for log in logs:
            if log.strip():
                print(log, file=sys.stderr)
    tmp = LIB + ".tmp"
    link = [cc, *ARCH, "-shared", "-o", tmp] + [o for _, o in jobs] + ["-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(flags_id)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
