"""Build ``libgde.so`` (the C ABI + sm_103a kernels) in-tree with nvcc.

Translation units compile in parallel, one ``-gencode`` (sm_103a only), and
link into ``faster-local-solver-for-gdes_gb300/build/libgde.so``.  A stamp of
the sources' mtimes and the flags skips the build when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG_DIR), "include")
BUILD = os.path.join(PKG_DIR, "build")
LIB = os.path.join(BUILD, "libgde.so")

SOURCES = ["push_engine.cu", "aux_kernels.cu", "plain.cu", "graph_edit.cu", "gde_capi.cu", "noalloc.cu", "spectral.cu", "sor_engine.cu",
           "probe.cu", "server.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
         "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgde.so")
    return exe


def _digest(extra_flags: list[str]) -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    h.update(" ".join(ARCH + FLAGS + extra_flags).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    # GDE_NVCC_EXTRA: extra nvcc flags (e.g. tuning macros) for experiments
    extra_flags = list(extra_flags or []) + os.environ.get("GDE_NVCC_EXTRA", "").split()
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "libgde.stamp")
    dig = _digest(extra_flags)
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    exe = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [exe, "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + FLAGS + extra_flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = [exe, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True,
                extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
