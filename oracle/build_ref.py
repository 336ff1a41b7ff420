"""Builds the reference's own CUDA operators into ``oracle/_ref/``.

The reference is a header-only CUDA C++ library (``include/curadon``) plus a
nanobind extension that cannot be built here (nanobind is not installed).
``ref_shim.cu`` repeats that extension's marshaling over the library and is
compiled with nvcc for sm_103a against the reference headers:

* where the reference tree exists (``CURADON_REF_ROOT``; unset, a checkout
  named ``reference`` beside this repository), the headers are used where
  they lie, and they are also
  staged, unmodified, into the git-ignored ``oracle/_ref/include`` -- the
  install step of a header-only library -- so that a machine without the
  reference tree can still compile the shim;
* otherwise the staged copy in ``oracle/_ref/include`` is used if present;
* otherwise nothing is built and the reference comparisons are skipped.

Nothing here is part of the product and ``oracle/_ref`` is never committed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REF_DIR = ORACLE_DIR / "_ref"
STAGED_INCLUDE = REF_DIR / "include"
OUT = REF_DIR / "libcuradon_ref.so"
SHIM = ORACLE_DIR / "ref_shim.cu"


def reference_include() -> Path | None:
    env = os.environ.get("CURADON_REF_ROOT")
    root = Path(env) if env else ORACLE_DIR.parent.parent / "reference"
    inc = root / "include"
    if (inc / "curadon" / "forward.hpp").exists():
        return inc
    return None


def stage(src_inc: Path) -> None:
    dst = STAGED_INCLUDE / "curadon"
    if dst.exists():
        shutil.rmtree(dst)
    shutil.copytree(src_inc / "curadon", dst)


def build(force: bool = False) -> Path | None:
    inc = reference_include()
    if inc is not None:
        REF_DIR.mkdir(exist_ok=True)
        stage(inc)
    elif (STAGED_INCLUDE / "curadon" / "forward.hpp").exists():
        inc = STAGED_INCLUDE
    else:
        return None
    if OUT.exists() and not force and OUT.stat().st_mtime > SHIM.stat().st_mtime:
        return OUT
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
           "--expt-extended-lambda", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-shared", f"-I{inc}", str(SHIM), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
        raise RuntimeError("building the reference shim failed")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
