"""In-tree build of the engine's shared libraries.

* ``lib/libsankhya_gb300.so``: the CUDA kernels (sm_103a only), the C++ host engine and the
  extern "C" boundary declared in include/sankhya_gb300.h. Built with nvcc directly, one
  translation unit per source, compiled in parallel.
* ``lib/liblpgen.so``: the synthetic LP generators (plain C).

Nothing is installed into site-packages; the libraries stay next to the sources so a fresh
machine only needs ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

from . import _paths

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["pdhg_kernels.cu", "mixed_kernels.cu", "batch_kernels.cu", "engine.cu", "layout.cu",
                "batch.cu", "qp_kernels.cu", "qp.cu", "capi.cu"]
HEADERS = ["common.cuh", "kernels.cuh", "tiles.cuh", "chunks.cuh", "decisions.cuh", "mixed.cuh",
           "batch.cuh", "qp.cuh", "qp_layout.hpp", "engine.hpp", "batch_engine.hpp",
           "qp_engine.hpp"]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + proc.stdout)
        raise RuntimeError(f"build step failed: {cmd[0]} ... {cmd[-1]}")
    return proc.stdout


def build_lpgen(force=False):
    src = os.path.join(_paths.LPGEN_DIR, "lpgen.c")
    os.makedirs(os.path.dirname(_paths.LPGEN_LIB), exist_ok=True)
    if force or _stale(_paths.LPGEN_LIB, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-o",
              _paths.LPGEN_LIB, src, "-lm"])
    return _paths.LPGEN_LIB


def build_engine(force=False, verbose_ptxas=False):
    """Compile every .cu for sm_103a and link the shared library."""
    out_dir = os.path.dirname(_paths.ENGINE_LIB)
    obj_dir = os.path.join(out_dir, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    headers = [os.path.join(_paths.CSRC_DIR, h) for h in HEADERS] + [
        os.path.join(_paths.INCLUDE_DIR, "sankhya_gb300.h")]
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
                    "-fvisibility=hidden", "-I", _paths.INCLUDE_DIR, "-I", _paths.CSRC_DIR,
                    "--expt-relaxed-constexpr"]
    if verbose_ptxas:
        flags += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        path = os.path.join(_paths.CSRC_DIR, src)
        obj = os.path.join(obj_dir, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append([NVCC] + flags + ["-c", path, "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if force or jobs or _stale(_paths.ENGINE_LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", _paths.ENGINE_LIB] + objs + ["-lcudart"])
    return "\n".join(logs)


def build_all(force=False):
    build_lpgen(force)
    build_engine(force)
