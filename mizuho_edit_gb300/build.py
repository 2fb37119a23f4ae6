"""In-tree build of libwpf_gb300.so (nvcc, sm_103a only).

The translation units compile in parallel and link into one shared library
under ``mizuho_edit_gb300/_build``; nothing is installed into site-packages.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from typing import List

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libwpf_gb300.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["wpf_capi.cu", "wpf_physics.cu", "wpf_solver.cu", "wpf_noalloc.cu", "wpf_net.cu",
           "wpf_ensemble.cu", "wpf_graph.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwpf_gb300")


def _deps() -> List[str]:
    out = [os.path.join(CSRC, s) for s in SOURCES]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        build_driver()
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    build_driver()
    return LIB_PATH


DRIVER_SRC = os.path.join(HERE, "host", "wpf_driver.cpp")
DRIVER_PATH = os.path.join(BUILD_DIR, "wpf_driver")


def build_driver() -> str:
    """The C++ host program (program main of the reference) on the C ABI."""
    if (os.path.exists(DRIVER_PATH) and os.path.getmtime(DRIVER_PATH) >= os.path.getmtime(DRIVER_SRC)
            and os.path.getmtime(DRIVER_PATH) >= os.path.getmtime(LIB_PATH)):
        return DRIVER_PATH
    cxx = shutil.which("g++") or "g++"
    tmp = DRIVER_PATH + f".tmp{os.getpid()}"
    cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, DRIVER_SRC, "-L", BUILD_DIR, "-lwpf_gb300",
           "-Wl,-rpath,$ORIGIN", "-pthread", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DRIVER_PATH)
    return DRIVER_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
