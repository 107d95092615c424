"""Build the CPU oracle (test infrastructure): oracle/_build/liborc.so and
oracle/_build/oracle_enumerate, plus the reference's own CPU solver via oracle/build_ref.sh,
from the reference tree where this machine has one ($PCA_REFERENCE_ROOT) or
from the copy oracle/stage_ref.sh staged in baseline/_ref/src (git-ignored).

    python oracle/build.py [--force]
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

ORACLE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(ORACLE, "_build")
# the reference tree, when this machine has one: $PCA_REFERENCE_ROOT
REFERENCE_ROOT = os.environ.get("PCA_REFERENCE_ROOT", "")
STAGED = os.path.join(os.path.dirname(ORACLE), "baseline", "_ref", "src")


def _newer(target: str, deps: list[str]) -> bool:
    return os.path.exists(target) and all(
        os.path.getmtime(d) <= os.path.getmtime(target) for d in deps)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, ".machine")
    if not os.path.exists(stamp) or open(stamp).read().strip() != platform.machine():
        force = True
    src = os.path.join(ORACLE, "pca_oracle.c")
    src2 = os.path.join(ORACLE, "oracle_levels.c")
    deps = [src, src2, os.path.join(ORACLE, "pca_oracle.h")]
    flags = ["-O2", "-std=c99", "-Wall", "-Wextra", "-pthread"]
    lib = os.path.join(BUILD, "liborc.so")
    cli = os.path.join(BUILD, "oracle_enumerate")
    procs = []
    if force or not _newer(lib, deps):
        procs.append(subprocess.Popen(["gcc", *flags, "-shared", "-fPIC", src, src2, "-o", lib]))
    cli_src = os.path.join(ORACLE, "oracle_cli.c")
    if force or not _newer(cli, deps + [cli_src]):
        procs.append(subprocess.Popen(["gcc", *flags, src, src2, cli_src, "-o", cli]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed")
    with open(stamp, "w") as f:
        f.write(platform.machine() + "\n")
    # the reference's own CPU solver: from the reference tree, else from the
    # sources oracle/stage_ref.sh staged (git-ignored) in baseline/_ref/src
    root = REFERENCE_ROOT if REFERENCE_ROOT and os.path.isdir(REFERENCE_ROOT) else STAGED
    ref_stamp = os.path.join(ORACLE, "_ref", ".machine")
    ref_ok = os.path.exists(os.path.join(ORACLE, "_ref", "enumerate")) and \
        os.path.exists(ref_stamp) and open(ref_stamp).read().strip() == platform.machine()
    if os.path.exists(os.path.join(root, "tools", "enumerate.c")) and (force or not ref_ok):
        subprocess.run(["sh", os.path.join(ORACLE, "build_ref.sh"), root],
                       check=True, capture_output=True)
    return lib


if __name__ == "__main__":
    print(build_oracle("--force" in sys.argv))
