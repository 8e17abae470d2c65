"""CPU oracle for the SynchRad radiation integral.

TEST INFRASTRUCTURE ONLY.  Nothing in ``synchrad_gb300`` imports this package:
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (and ``--impl reference``) load it, and only as the checker or the timed
CPU baseline.

Two interchangeable back ends with the same C ABI:

* ``port``: ``oracle/sr_oracle.c``, a plain-C restatement of the reference's
  eight OpenCL kernels (``synchrad/kernel_farfield.cl``,
  ``synchrad/kernel_nearfield.cl``), FP64 and FP32.  Builds anywhere with gcc.
* ``ref``: the reference's own kernel source compiled for the CPU through
  ``oracle/ref_shim.hpp`` (``oracle/build_ref.sh`` -> ``oracle/_ref/``).  Only
  buildable where the reference source tree is present.

The host-side logic of ``synchrad/calc.py`` (grid, device axes, snapshot
iterations, per-track ``it_range`` handling, layout swap, weight
normalisation) is restated in :mod:`oracle.host`.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
REF_DIR = HERE / "_ref"
PORT_LIB = BUILD_DIR / "libsr_oracle.so"
REF_LIB = REF_DIR / "libsr_ref.so"
REFERENCE_ROOT = Path(os.environ.get("SR_REFERENCE_ROOT", "/root/reference"))

COMP_IDS = {
    "total": 0,
    "cartesian": 1,
    "cartesian_complex": 2,
    "spheric": 3,
    "spheric_complex": 4,
}


def build_port(force: bool = False) -> Path:
    """Compile oracle/sr_oracle.c into oracle/_build/libsr_oracle.so."""
    src = HERE / "sr_oracle.c"
    deps = [src, HERE / "sr_oracle_impl.h"]
    if (not force and PORT_LIB.exists()
            and all(PORT_LIB.stat().st_mtime >= d.stat().st_mtime for d in deps)):
        return PORT_LIB
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = PORT_LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fopenmp", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, PORT_LIB)
    return PORT_LIB


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference kernels (needs the reference source tree)."""
    if not (REFERENCE_ROOT / "synchrad" / "kernel_farfield.cl").exists():
        return REF_LIB if REF_LIB.exists() else None
    deps = [HERE / "ref_shim.hpp", HERE / "ref_driver.cpp", HERE / "build_ref.sh"]
    if (not force and REF_LIB.exists()
            and all(REF_LIB.stat().st_mtime >= d.stat().st_mtime for d in deps)):
        return REF_LIB
    subprocess.run(["bash", str(HERE / "build_ref.sh"), str(REFERENCE_ROOT)],
                   check=True, stdout=subprocess.DEVNULL)
    return REF_LIB


_libs: dict[str, ctypes.CDLL] = {}


def _bind(lib: ctypes.CDLL, far_name: str, near_name: str) -> None:
    vp = ctypes.c_void_p
    u32 = ctypes.c_uint32
    far = getattr(lib, far_name)
    far.restype = ctypes.c_int
    far.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp),
                    ctypes.POINTER(vp), ctypes.c_double, u32, u32, u32,
                    ctypes.POINTER(vp), u32, u32, u32, ctypes.c_double, u32,
                    ctypes.POINTER(u32), vp, ctypes.c_int]
    near = getattr(lib, near_name)
    near.restype = ctypes.c_int
    near.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp),
                     ctypes.POINTER(vp), ctypes.c_double, u32, u32, u32,
                     ctypes.POINTER(vp), ctypes.c_double, u32, u32, u32,
                     ctypes.c_double, u32, ctypes.POINTER(u32), vp,
                     ctypes.c_int]
    lib.sr_far_fn = far
    lib.sr_near_fn = near


def load(kind: str = "port") -> ctypes.CDLL:
    """Load the ``port`` (C restatement) or ``ref`` (reference source) oracle."""
    if kind in _libs:
        return _libs[kind]
    if kind == "port":
        lib = ctypes.CDLL(str(build_port()))
        _bind(lib, "sro_far", "sro_near")
    elif kind == "ref":
        path = build_ref()
        if path is None or not path.exists():
            raise FileNotFoundError("reference kernels are not available here")
        lib = ctypes.CDLL(str(path))
        _bind(lib, "sr_ref_far", "sr_ref_near")
    else:
        raise ValueError(kind)
    _libs[kind] = lib
    return lib


def ref_available() -> bool:
    try:
        load("ref")
        return True
    except (FileNotFoundError, OSError, subprocess.CalledProcessError):
        return False


def _ptrs(arrays):
    arr = (ctypes.c_void_p * len(arrays))()
    for i, a in enumerate(arrays):
        arr[i] = None if a is None else a.ctypes.data
    return arr


def run_track(kind: str, mode: str, comp: str, spectra, track6, wp, it_start,
              it_end, n_steps, axes, grid_n, dt, it_snaps, form_factor=None,
              L_screen=0.0, nthreads: int | None = None) -> None:
    """One reference kernel launch (one track) on the CPU, accumulating in place.

    ``spectra``: list of contiguous arrays in device order
    ``[nSnaps][nPhi][nTheta|nR][nOmega]``, all of the track's dtype.
    """
    lib = load(kind)
    dtype = spectra[0].dtype
    dt_id = 0 if dtype == np.float64 else 1
    for a in list(spectra) + list(track6) + list(axes):
        assert a.dtype == dtype and a.flags.c_contiguous
    sp = list(spectra) + [None] * (6 - len(spectra))
    snaps = np.ascontiguousarray(it_snaps, dtype=np.uint32)
    nth = nthreads or os.cpu_count() or 1
    ff = None if form_factor is None else np.ascontiguousarray(form_factor, dtype=dtype)
    if mode == "far":
        rc = lib.sr_far_fn(dt_id, COMP_IDS[comp], _ptrs(sp), _ptrs(track6),
                           float(wp), int(it_start), int(it_end), int(n_steps),
                           _ptrs(axes), *map(int, grid_n), float(dt),
                           len(snaps), snaps.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                           None if ff is None else ff.ctypes.data, nth)
    else:
        rc = lib.sr_near_fn(dt_id, COMP_IDS[comp], _ptrs(sp), _ptrs(track6),
                            float(wp), int(it_start), int(it_end), int(n_steps),
                            _ptrs(axes), float(L_screen), *map(int, grid_n),
                            float(dt), len(snaps),
                            snaps.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                            None if ff is None else ff.ctypes.data, nth)
    if rc != 0:
        raise ValueError(f"oracle rejected the launch arguments (rc={rc})")
