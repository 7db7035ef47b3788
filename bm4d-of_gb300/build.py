"""In-tree build of libbm4dof_gpu.so for GB300 (sm_103a) with nvcc.

    python bm4d-of_gb300/build.py          # or: import build; build.build()

Every translation unit is compiled in parallel to an object file, then linked
into lib/libbm4dof_gpu.so.  Device code is compiled with --fmad=false: the
exact path keeps every multiply and add separately rounded, as the reference
computes them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libbm4dof_gpu.so")
CLI = os.path.join(OUT, "bm4dof")          # the command line, linked to LIB
TVL1_CLI = os.path.join(OUT, "tvl1flow")   # the optical-flow command line, linked to LIB
CLI_ALIAS = os.path.join(OUT, "bm4d-of")   # the name the reference's scripts call the CLI by
AWGN_CLI = os.path.join(OUT, "awgn")       # noise and PSNR tools of the reference's scripts (host only)
PSNR_CLI = os.path.join(OUT, "psnr")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
SOURCES = ["search.cu", "search_vbm3d.cu", "search_tc.cu", "filter.cu", "aggregate.cu", "runtime.cu", "noalloc.cu",
           "mlp.cu", "learned.cu", "tvl1.cu", "peaks.cu",
           "params.cpp", "basis.cpp"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(SRC, src)
    deps = [path] + [os.path.join(SRC, h) for h in os.listdir(SRC)
                     if h.endswith((".cuh", ".hpp", ".h")) and h != "frames.hpp"]
    deps.append(os.path.join(HERE, "..", "include", "bm4dof.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + NVFLAGS + ["-x", "cu" if src.endswith(".cu") else "c++", "-c", path, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def _link_cli(main_src: str, exe: str, gpu: bool = True) -> None:
    """A command line: main_src plus the frame files, host code only, linked
    to LIB when gpu (no contraction, so that double arithmetic such as the
    colour reduction rounds alike on every host)."""
    src = [os.path.join(SRC, main_src), os.path.join(SRC, "frames.cpp")]
    deps = src + [os.path.join(SRC, "frames.hpp"), os.path.join(HERE, "..", "include", "bm4dof.h")]
    deps += [LIB] if gpu else []
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(x) for x in deps):
        return
    cxx = shutil.which("g++") or "g++"
    link = ["-L" + OUT, "-lbm4dof_gpu", "-Wl,-rpath,$ORIGIN"] if gpu else []
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", *src, "-o", exe, *link]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} build failed:\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(lambda a: _link_cli(*a), [("cli.cpp", CLI), ("tvl1_cli.cpp", TVL1_CLI),
                                               ("awgn_cli.cpp", AWGN_CLI, False),
                                               ("psnr_cli.cpp", PSNR_CLI, False)]))
    if not os.path.lexists(CLI_ALIAS):
        os.symlink(os.path.basename(CLI), CLI_ALIAS)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
