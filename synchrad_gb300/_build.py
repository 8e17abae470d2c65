"""Build recipe of the in-tree CUDA library ``synchrad_gb300/libsynchrad_gb300.so``.

Every translation unit is compiled for sm_103a only (GB300), in parallel, with
nvcc; the objects go to ``synchrad_gb300/_build/`` and the shared library next
to this file.  ``sr_port.cu`` (the plain ports of the reference kernels) is
compiled with ``--fmad=false`` so that each product and sum rounds on its own,
as in the reference built without contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsynchrad_gb300.so"
INCLUDE = PKG.parent / "include"

SOURCES = {
    "sr_api.cu": [],
    "sr_port.cu": ["--fmad=false"],
    "sr_far_mixed.cu": [],
    "sr_far_df.cu": [],
    "sr_near_mixed.cu": [],
    "sr_far_adjoint.cu": [],
    "sr_diag.cu": [],
    "sr_noalloc.cu": [],
    "sr_tune.cu": [],
    "sr_near_adjoint.cu": [],
}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
          "--expt-relaxed-constexpr", "-I", str(INCLUDE)]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build synchrad_gb300")
    return cand


def _deps():
    return ([CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
            + [INCLUDE / "synchrad_gb300.h", Path(__file__)])


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(item):
        src, extra = item
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 1)) as ex:
        results = list(ex.map(compile_one, SOURCES.items()))
    if verbose:
        for _, log in results:
            print(log)
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
