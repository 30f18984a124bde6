"""Builds the native parts of smatranem_gb300 in-tree.

Outputs (git-ignored) under smatranem_gb300/_build/:
  libsmatran_fdtd.so   the C ABI of include/smatran_fdtd.h (CUDA kernels for
                       sm_103a + host precompute + deck I/O)
  FDTD                 the drop-in command-line solver (reads input.txt and the
                       Data/ files of the SMatrAnEM mesher chain)
  Scalc                the drop-in S-matrix program (same input.txt, Med, Mode
                       and Xi files as SMatrAnEM's Scalc; writes _Smatrix.dat)

Only nvcc and gcc are used, one -gencode (sm_103a), translation units compiled
in parallel.  Run ``python -m smatranem_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libsmatran_fdtd.so")
EXE = os.path.join(OUT, "FDTD")
SCALC_EXE = os.path.join(OUT, "Scalc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host C: the reference's flags (-O2 -std=c11) plus no FMA contraction, so the
# FP64 precompute rounds exactly as the reference does on the same host
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-Wall", "-I" + INC, "-I" + CSRC]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CSRC,
                  "-Xptxas", "-v"]
# per-file extras: the FP64 path must not fuse multiply-adds (bit-identical results)
NV_EXTRA = {"fdtd_f64.cu": ["-fmad=false"]}

C_SOURCES = ["host_precompute.c", "errors.c", "deck_io.c"]
CU_SOURCES = ["fdtd_f64.cu", "fdtd_f32.cu", "fdtd_plan.cu", "fdtd_overlap.cu", "fdtd_adjoint.cu",
              "fdtd_group.cu", "mode_solver.cu", "dense_z.cu", "zgemm_tc.cu", "scalc.cu", "fdtd_row32.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build smatranem_gb300")


def _run(cmd, log):
    r = subprocess.run(cmd, capture_output=True, text=True)
    log.append((cmd, r.stdout + r.stderr))
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile everything that is out of date; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INC, "smatran_fdtd.h"))
    jobs, objs = [], []
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["gcc"] + CFLAGS + ["-c", s, "-o", o])
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVFLAGS + NV_EXTRA.get(src, []) + ["-c", s, "-o", o])
    log = []
    with cf.ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        for f in [ex.submit(_run, j, log) for j in jobs]:
            f.result()
    if force or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lm", "-lpthread"], log)
    main_c = os.path.join(CSRC, "fdtd_main.c")
    if os.path.exists(main_c) and (force or _stale(EXE, [main_c, LIB] + headers)):
        _run(["gcc"] + CFLAGS + [main_c, "-o", EXE, "-L" + OUT, "-lsmatran_fdtd", "-Wl,-rpath,$ORIGIN", "-lm"], log)
    cli_c = os.path.join(CSRC, "scalc_cli.c")
    if os.path.exists(cli_c) and (force or _stale(SCALC_EXE, [cli_c, LIB] + headers)):
        _run(["gcc"] + CFLAGS + [cli_c, "-o", SCALC_EXE, "-L" + OUT, "-lsmatran_fdtd", "-Wl,-rpath,$ORIGIN", "-lm"],
             log)
    if verbose:
        for cmd, out in log:
            print(" ".join(cmd))
            if out.strip():
                print(out)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
