"""Builds the native library ``cloverleaf_gb300/_lib/libep_gb300.so`` in-tree.

CUDA translation units are compiled for sm_103a only (one ``-gencode``) in
parallel with the host C++ unit; a source/flag hash stamp skips rebuilds.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libep_gb300.so")

CU_SOURCES = ("ep_fwd.cu", "ep_sort.cu", "ep_red.cu", "ep_ctx.cu", "ep_knn.cu")
CPP_SOURCES = ("ep_host.cpp",)
HEADERS = ("ep_internal.h", "ep_device.cuh", "ep_launch.cuh")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I" + INCLUDE]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cloverleaf_gb300")


def _stamp() -> str:
    h = hashlib.sha256()
    for name in CU_SOURCES + CPP_SOURCES + HEADERS:
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode() + f.read())
    for name in sorted(os.listdir(INCLUDE)):
        with open(os.path.join(INCLUDE, name), "rb") as f:
            h.update(name.encode() + f.read())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles and links the library if sources changed; returns its path."""
    stamp_path = os.path.join(LIB_DIR, ".stamp")
    stamp = _stamp()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp_path):
        with open(stamp_path) as f:
            if f.read().strip() == stamp:
                return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        jobs.append(([nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj], obj))
    for src in CPP_SOURCES:
        obj = os.path.join(OBJ_DIR, src.replace(".cpp", ".o"))
        jobs.append((["g++"] + CXX_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj], obj))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(lambda j: run(j[0]), jobs))
    tmp = LIB_PATH + ".tmp"
    run([nvcc, "-shared", ARCH, "-o", tmp] + [j[1] for j in jobs] + ["-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB_PATH)
    with open(stamp_path, "w") as f:
        f.write(stamp)
    return LIB_PATH
