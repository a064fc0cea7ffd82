"""Build libcryoim_gb300.so (sm_103a) and the CPU oracle, in-tree.

The CUDA library is compiled with nvcc directly (no torch extension: the C ABI in
include/cryoim.h carries no torch types).  Translation units:

* prep.cu  -- -fmad=false: FP32 expressions round where the Fortran reference rounds;
* score.cu -- hot scoring kernels, multiply-add contraction allowed;
* api.cu   -- context, drivers, C ABI (host code built with -ffp-contract=off);
* fsc.cu   -- -fmad=false: half-map FSC and the FSC-weighted map;
* mapops.cu -- -fmad=false: real-space icosahedral average, merge output step;
* center.cu -- -fmad=false: origin centring of icosprocess mode 3;
* local.cu -- -fmad=false: local_refine's sub-particle refinement;
* learn.cu -- the learned orientation proposer (features, CNN forward / backward, Adam);
* conv_tc.cu -- the proposer's convolutions on the tcgen05 tensor cores (TF32);
* io.cpp, local_host.cpp -- host only (g++): MRC / orientation / tnf files, local_box
  geometry and local_refine parameters.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIBNAME = "libcryoim_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n  " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.stderr.strip():
        sys.stderr.write(r.stderr)


UNITS = {
    "prep.cu": ["-fmad=false"],
    "score.cu": [],
    "api.cu": [],
    "noalloc.cu": [],
    "gemm_tc.cu": [],
    "contract.cu": [],
    "fsc.cu": ["-fmad=false"],
    "mapops.cu": ["-fmad=false"],
    "center.cu": ["-fmad=false"],
    "local.cu": ["-fmad=false"],
    "learn.cu": [],
    "conv_tc.cu": [],
}


def build_library(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I", os.path.join(ROOT, "include")] + (extra or [])
    objs = []
    cmds = []
    for src, flags in UNITS.items():
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(obj)
        cmds.append([nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + common + flags)
    for src in HOST_UNITS:
        obj = os.path.join(OUT, src.replace(".cpp", ".o"))
        objs.append(obj)
        cmds.append([cxx(), "-c", os.path.join(CSRC, src), "-o", obj, "-O2", "-std=c++17", "-fPIC",
                     "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include")])
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(_run, cmds))
    lib = os.path.join(OUT, LIBNAME)
    _run([nvcc(), "-shared", "-o", lib] + objs + ARCH + ["-lcufft", "-lcudart"])
    if verbose:
        print("built", lib)
    build_tools(lib)
    return lib


HOST_UNITS = ["io.cpp", "local_host.cpp"]
TOOLS = {"icosprocess": "icosprocess.cpp", "proc_icos": "proc_icos.cpp",
         "merge_icosprocess_subrec": "merge_subrec.cpp", "local_box": "local_box.cpp",
         "local_refine": "local_refine.cpp"}
BIN = os.path.join(HERE, "bin")


def cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def build_tools(lib: str) -> None:
    """The drop-in executables (C++ hosts over the C ABI), rpath to the in-tree library."""
    os.makedirs(BIN, exist_ok=True)
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    cmds = []
    for name, src in TOOLS.items():
        path = os.path.join(CSRC, "host", src)
        if not os.path.exists(path):
            continue
        cmds.append([cxx(), "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", path, "-o",
                     os.path.join(BIN, name), "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                     "-L", OUT, "-lcryoim_gb300", "-Wl,-rpath,$ORIGIN/../_lib"])
    with ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        list(ex.map(_run, cmds))


def build_oracle() -> str:
    """The CPU oracle (test infrastructure; never linked into the library)."""
    odir = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", odir])
    return os.path.join(odir, "_build", "libcryoim_oracle.so")


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, verbose)
        f2 = ex.submit(build_oracle)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(verbose=True)
