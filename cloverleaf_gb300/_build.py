"""Builds the native libraries in-tree, under ``cloverleaf_gb300/_lib/``.

* ``libep_gb300.so``: the trainer.  CUDA translation units are compiled for
  sm_103a only (one ``-gencode``) in parallel with the host C++ unit.
* ``libep_datagen.so``: the synthetic workload generators (host C++ only),
  kept apart so that the benchmark's CPU reference arm can generate its
  workload without loading the trainer.

A source/flag hash stamp per library skips rebuilds.
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
DATAGEN_PATH = os.path.join(LIB_DIR, "libep_datagen.so")
DATAGEN_SOURCES = ("ep_datagen.cpp",)

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


def _stamp(sources) -> str:
    h = hashlib.sha256()
    for name in sources:
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode() + f.read())
    for name in sorted(os.listdir(INCLUDE)):
        with open(os.path.join(INCLUDE, name), "rb") as f:
            h.update(name.encode() + f.read())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _fresh(path: str, stamp: str) -> bool:
    stamp_path = path + ".stamp"
    if not (os.path.exists(path) and os.path.exists(stamp_path)):
        return False
    with open(stamp_path) as f:
        return f.read().strip() == stamp


def _run(cmd, verbose: bool):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_datagen(verbose: bool = False, force: bool = False) -> str:
    """Compiles and links libep_datagen.so if its sources changed; returns its path."""
    stamp = _stamp(DATAGEN_SOURCES)
    if not force and _fresh(DATAGEN_PATH, stamp):
        return DATAGEN_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    tmp = DATAGEN_PATH + ".tmp"
    _run(["g++"] + CXX_FLAGS + ["-shared", "-o", tmp] + [os.path.join(CSRC, s) for s in DATAGEN_SOURCES] + ["-lgomp"],
         verbose)
    os.replace(tmp, DATAGEN_PATH)
    with open(DATAGEN_PATH + ".stamp", "w") as f:
        f.write(stamp)
    return DATAGEN_PATH


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles and links the trainer library (and the generator library) if
    sources changed; returns the trainer library's path."""
    build_datagen(verbose, force)
    stamp = _stamp(CU_SOURCES + CPP_SOURCES + HEADERS)
    if not force and _fresh(LIB_PATH, stamp):
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

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(lambda j: _run(j[0], verbose), jobs))
    tmp = LIB_PATH + ".tmp"
    _run([nvcc, "-shared", ARCH, "-o", tmp] + [j[1] for j in jobs] + ["-Xcompiler", "-fopenmp", "-lgomp"], verbose)
    os.replace(tmp, LIB_PATH)
    with open(LIB_PATH + ".stamp", "w") as f:
        f.write(stamp)
    return LIB_PATH
