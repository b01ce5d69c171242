"""Build libpfgb.so in-tree with nvcc (sm_103a only).

``python -m pyflow_solver_gb300._build`` or ``__graft_entry__.build()``.
The translation units compile in parallel; the shared library lands in
``pyflow_solver_gb300/_lib/libpfgb.so`` (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libpfgb.so")
SOURCES = ["step64.cu", "mixed.cu", "ops.cu", "krylov.cu", "capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-fvisibility=hidden"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpfgb.so")


def _deps_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(os.path.dirname(HERE), "include", "pfgb.h")
    return os.path.exists(hdr) and os.path.getmtime(hdr) > t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _deps_newer(LIB):
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    nv = nvcc()
    with tempfile.TemporaryDirectory(prefix="pfgb_build_") as tmp:
        procs = []
        objs = []
        for src in SOURCES:
            obj = os.path.join(tmp, src.replace(".cu", ".o"))
            objs.append(obj)
            cmd = [nv, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        for cmd, p in procs:
            out, _ = p.communicate()
            if p.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{out.decode(errors='replace')}")
            if verbose and out:
                sys.stdout.write(out.decode(errors="replace"))
        tmp_lib = os.path.join(tmp, "libpfgb.so")
        link = [nv, *ARCH, "-shared", "-o", tmp_lib, *objs]
        r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout.decode(errors='replace')}")
        shutil.move(tmp_lib, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
