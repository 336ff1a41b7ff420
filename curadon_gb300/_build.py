"""Builds the sm_103a shared library ``libcuradon_gb300.so`` in-tree.

Every ``csrc/*.cu`` file is compiled by its own ``nvcc`` process (in
parallel) for ``sm_103a`` only, then linked into one shared library next to
this file.  No CMake; the compile is a few seconds per translation unit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = REPO_DIR / "_build"
LIB_NAME = "libcuradon_gb300.so"
LIB_PATH = PKG_DIR / LIB_NAME

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and (Path(root) / "bin" / "nvcc").exists():
            return str(Path(root) / "bin" / "nvcc")
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build curadon_gb300")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def needs_build() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    """Compile and link the library if any source changed (or ``force``)."""
    if not force and not needs_build():
        return LIB_PATH
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    objs = []
    cmds = []
    for src in _sources():
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        cmds.append([nvcc, *NVCC_FLAGS, *ARCH_FLAGS, *extra_flags, f"-I{INCLUDE}", f"-I{CSRC}",
                     "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        logs = list(ex.map(_run, cmds))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    _run([nvcc, "-shared", *ARCH_FLAGS, "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True))
