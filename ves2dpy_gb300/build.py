"""Build the C-ABI shared library ``_lib/libves2d_gb300.so`` with nvcc.

One translation unit per stage, compiled in parallel for sm_103a only, then
linked with the CUDA runtime into a self-contained ``.so`` whose exported
symbols are exactly the ``extern "C"`` functions of ``include/ves2d_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libves2d_gb300.so")
SOURCES = ["ves_ctx.cu", "ves_spectral.cu", "ves_blas.cu", "ves_alpert.cu", "ves_farfield.cu",
           "ves_farfield_mp.cu", "ves_near.cu", "ves_step.cu", "ves_capi.cu", "ves_noalloc.cu", "ves_post.cu",
           "ves_nets.cu", "ves_nets_tc.cu", "ves_mlarm.cu", "ves_traj.cu",
           "ves_repulsion.cu", "ves_rbf.cu", "ves_dl.cu", "ves_targets.cu", "ves_train.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-diag-suppress", "550"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _needs(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "ves2d_gb300.h"))
    cc = nvcc()
    extra = os.environ.get("VES2D_NVCC_EXTRA", "").split()
    jobs = []
    objs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _needs(obj, [sp] + headers):
            cmd = [cc, *ARCH, *FLAGS, *extra, "-I", os.path.join(ROOT, "include"), "-c", sp, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    if jobs or force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lrt", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
