"""Build the GB300 engine in-tree: libcipsi_gb300.so and the cip_gpu,
moy_gpu and bd_gpu drop-ins.

Sources are compiled for sm_103a only, in parallel, and skipped when the
sources and flags have not changed since the last build.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcipsi_gb300.so")
EXE = os.path.join(OUT, "cip_gpu")
MOY_EXE = os.path.join(OUT, "moy_gpu")
BD_EXE = os.path.join(OUT, "bd_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# no fused multiply-add contraction in host code: the same results on x86 and Arm
CXXFLAGS = ["-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-Wall"]

CU_SOURCES = ["cipsi_engine.cu", "pt2_w1.cu", "pt2_w2.cu", "pt2_adj.cu", "pt2_adj_w2.cu", "hbuild.cu", "davidson.cu"]
HOST_SOURCES = ["cip_host.cpp", "moy_host.cpp", "bd_host.cpp"]
MAINS = {"cip_gpu": "cip_gpu_main.cpp", "moy_gpu": "moy_gpu_main.cpp", "bd_gpu": "bd_gpu_main.cpp"}
SOURCES = CU_SOURCES + HOST_SOURCES + list(MAINS.values()) + ["pt2_common.cuh", "pt2_kernel.cuh", "host_io.h",
                                                              "symeig.h"]
HEADERS = [os.path.join(ROOT, "include", "cipsi_gb300.h")]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _digest(extra: str = "") -> str:
    h = hashlib.sha256()
    for f in [os.path.join(CSRC, s) for s in SOURCES] + HEADERS + [os.path.abspath(__file__)]:
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(extra.encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    stamp = os.path.join(OUT, ".stamp")
    dig = _digest(" ".join(ARCH + NVFLAGS + CXXFLAGS))
    if (not force and os.path.exists(LIB) and all(os.path.exists(os.path.join(OUT, e)) for e in MAINS)
            and os.path.exists(stamp)):
        if open(stamp).read().strip() == dig:
            return LIB
    objs = {c: os.path.join(OUT, c.replace(".cu", ".o")) for c in CU_SOURCES}
    for c in HOST_SOURCES + list(MAINS.values()):
        objs[c] = os.path.join(OUT, c.replace(".cpp", ".o"))
    jobs = [[nvcc] + ARCH + NVFLAGS + ["-Xptxas", "-v", "-c", os.path.join(CSRC, c), "-o", objs[c]]
            for c in CU_SOURCES]
    jobs += [["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, c), "-o", objs[c]]
             for c in HOST_SOURCES + list(MAINS.values())]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    ptxas = "".join(outs[:len(CU_SOURCES)])
    if verbose:
        sys.stdout.write(ptxas)
    with open(os.path.join(OUT, "ptxas_info.txt"), "w") as fh:
        fh.write(ptxas)
    _run([nvcc] + ARCH + ["-shared", "-o", LIB] + [objs[c] for c in CU_SOURCES + HOST_SOURCES] + ["-lcudart"])
    for exe, main in MAINS.items():
        _run(["g++", "-o", os.path.join(OUT, exe), objs[main], "-L" + OUT, "-lcipsi_gb300", "-Wl,-rpath,$ORIGIN",
              "-L" + os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64"), "-lcudart"])
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
