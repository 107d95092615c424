"""Build recipe for the native parts: libpcagb.so (CUDA engine + libpca ABI)
and the solver CLIs linked against it.

    python -m pca_gb300.build [--force]

Compiles for sm_103a only. Translation units build in parallel; no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pca_gb300", "csrc")
LIBDIR = os.path.join(ROOT, "pca_gb300", "_lib")
OBJDIR = os.path.join(ROOT, "pca_gb300", "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra"]

CU_SOURCES = ["engine.cu", "noalloc.cu", "valuenet.cu", "valuenet_tc.cu", "branch.cu", "server.cu"]
CXX_SOURCES = ["host_abi.cpp"]
CLI_SOURCES = {"enumerate": "cli_enumerate.cpp", "gpu_hybrid": "cli_gpu_hybrid.cpp"}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", "pca_gb300.h")]


def build_engine(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    # objects built on another machine type (x86 vs aarch64) are never reused
    stamp = os.path.join(LIBDIR, ".machine")
    here = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != here:
        force = True
    nv = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            jobs.append([nv, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            jobs.append(["g++", *CXX_FLAGS, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    lib = os.path.join(LIBDIR, "libpcagb.so")
    if force or jobs or not _newer(lib, objs):
        _run([nv, *ARCH, "-shared", "-o", lib, *objs, "-lpthread"])
    cli_jobs = []
    for name, src in CLI_SOURCES.items():
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        exe = os.path.join(LIBDIR, name)
        if force or not _newer(exe, [s, lib] + hdrs):
            cli_jobs.append(["g++", *CXX_FLAGS, s, "-o", exe, "-L" + LIBDIR, "-lpcagb",
                             "-Wl,-rpath,$ORIGIN"])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(cli_jobs))) as ex:
        list(ex.map(_run, cli_jobs))
    with open(stamp, "w") as f:
        f.write(here + "\n")
    return lib


def main(argv: list[str]) -> None:
    force = "--force" in argv
    print(build_engine(force))


if __name__ == "__main__":
    main(sys.argv[1:])
