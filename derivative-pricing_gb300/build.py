"""Build recipe for libmcd_gpu.so (sm_103a) and the C++20 drop-in shim.

Compiles every csrc/*.cu with nvcc for sm_103a only, every csrc/*.cpp with
g++ (C++20, ISO mode, no FP contraction, matching the reference's flags), in
parallel, and links one shared library into ``build/``.  The C++ shim
(``cpp/``: mcd::pricers signatures over the C ABI, and the JSON CLI) links
against that library.

    python derivative-pricing_gb300/build.py [--force] [-v]
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CPP = os.path.join(PKG, "cpp")
BUILD = os.path.join(PKG, "build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libmcd_gpu.so")
SHIM_LIB = os.path.join(BUILD, "libmcd_shim.so")
CLI = os.path.join(BUILD, "mcd_gpu_cli")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _digest(paths, extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    return h.hexdigest()


def _headers():
    out = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    return out


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return r


def nvcc_flags(src: str):
    flags = ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
             "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC] + ARCH
    # Per-file flags: a "// nvcc-flags: ..." line in the source's leading
    # comment block (read up to the first line that is neither a comment nor blank).
    with open(src) as f:
        for line in f.read().splitlines():
            if line.startswith("// nvcc-flags:"):
                flags += line.split(":", 1)[1].split()
            elif line.strip() and not line.lstrip().startswith("//"):
                break
    extra = os.environ.get("MCD_NVCC_FLAGS")
    if extra:
        flags += extra.split()
    return flags


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link; returns the path of libmcd_gpu.so.  Incremental by content hash."""
    os.makedirs(BUILD, exist_ok=True)
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    cc = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cpp"))
    shim = sorted(os.path.join(CPP, f) for f in os.listdir(CPP) if f.endswith((".cpp", ".hpp"))) \
        if os.path.isdir(CPP) else []
    stamp = os.path.join(BUILD, ".stamp")
    digest = _digest(cu + cc + shim + _headers() + [__file__],
                     " ".join(ARCH) + os.environ.get("MCD_NVCC_FLAGS", ""))
    if (not force and os.path.exists(LIB) and os.path.exists(stamp)
            and open(stamp).read() == digest):
        return LIB
    nvcc = _nvcc()
    cuda = _cuda_home()
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        jobs.append([nvcc, "-c", src, "-o", obj] + nvcc_flags(src))
    for src in cc:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        jobs.append(["g++", "-std=c++20", "-O3", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
                     "-I", CSRC, "-I", os.path.join(cuda, "include"), "-c", src, "-o", obj])
    workers = min(len(jobs), os.cpu_count() or 4) or 1
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for fut in [ex.submit(_run, j, verbose) for j in jobs]:
            fut.result()
    _run([nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-cudart", "shared",
          "-Xlinker", "-rpath," + os.path.join(cuda, "lib64"), "-lcuda"], verbose)
    if shim:
        _build_shim(verbose)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


def _build_shim(verbose: bool) -> None:
    srcs = sorted(os.path.join(CPP, f) for f in os.listdir(CPP) if f.endswith(".cpp") and f != "mcd_gpu_cli.cpp")
    if srcs:
        _run(["g++", "-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-shared", "-I", INCLUDE,
              "-I", CPP, "-o", SHIM_LIB] + srcs + ["-L", BUILD, "-lmcd_gpu",
              "-Wl,-rpath,$ORIGIN"], verbose)
    cli = os.path.join(CPP, "mcd_gpu_cli.cpp")
    if os.path.exists(cli):
        _run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-I", INCLUDE, "-I", CPP, "-o", CLI,
              cli, "-L", BUILD, "-lmcd_shim", "-lmcd_gpu", "-Wl,-rpath,$ORIGIN"], verbose)


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
