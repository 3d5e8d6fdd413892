"""Build the in-tree CUDA library ``picongpu_gb300/_build/libpicgb.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by its own nvcc process (in
parallel), then linked into one shared library with a static CUDA runtime.
Usage: ``python -m picongpu_gb300.build [--force] [--debug]``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpicgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpicgb.so")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps() -> list[str]:
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "picgb.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps() + [__file__])


def build(force: bool = False, debug: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    common = ARCH + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler", "-fPIC",
        "-I", os.path.join(ROOT, "include"),
        "-I", CSRC,
        "--expt-relaxed-constexpr",
    ]
    if debug:
        common += ["-DPICGB_DEBUG"]
    # tuning knobs, e.g. PICGB_NVCC_DEFINES="PICGB_PUSH_MIN_BLOCKS=2"
    for d in os.environ.get("PICGB_NVCC_DEFINES", "").split():
        common += [f"-D{d}"]
    if verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = [cc, *common, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, debug="--debug" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
