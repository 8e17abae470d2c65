"""ctypes binding of the C ABI in include/synchrad_gb300.h.

The shared library is built in-tree (``synchrad_gb300/libsynchrad_gb300.so``,
see :mod:`synchrad_gb300._build`).  There is no fallback: if the library is
missing or fails to load, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import _build

SR_OK = 0
SR_ERR_INVALID = -1
SR_ERR_UNSUPPORTED = -2
SR_ERR_CUDA = -3
SR_ERR_WORKSPACE = -4
SR_ERR_TIMEOUT = -5

SR_DTYPE_F64 = 0
SR_DTYPE_F32 = 1
SR_MODE_FAR = 0
SR_MODE_NEAR = 1

COMP_IDS = {
    "total": 0,
    "cartesian": 1,
    "cartesian_complex": 2,
    "spheric": 3,
    "spheric_complex": 4,
}
N_OUT = {0: 1, 1: 3, 2: 6, 3: 3, 4: 6}

SR_PREC_DOUBLE = 0
SR_PREC_FLOAT = 1
SR_PREC_FLOAT_NATIVE = 2
SR_PREC_MIXED = 3
SR_PREC_DF = 4


class SynchRadError(RuntimeError):
    """A failure reported by the CUDA library (code + sr_last_error message)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"synchrad_gb300 error {code}: {message}")
        self.code = code


class SrTracks(ctypes.Structure):
    _fields_ = [
        ("n_tracks", ctypes.c_uint32),
        ("dtype", ctypes.c_uint32),
        ("total_steps", ctypes.c_int64),
        ("offsets", ctypes.c_void_p),
        ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
        ("ux", ctypes.c_void_p), ("uy", ctypes.c_void_p), ("uz", ctypes.c_void_p),
        ("weight", ctypes.c_void_p),
        ("it_start", ctypes.c_void_p),
        ("it_end", ctypes.c_void_p),
        ("snap_its", ctypes.c_void_p),
        ("snap_stride", ctypes.c_uint32),
        ("n_snaps", ctypes.c_uint32),
        ("dt", ctypes.c_double),
    ]


class SrGrid(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_uint32),
        ("dtype", ctypes.c_uint32),
        ("n_omega", ctypes.c_uint32),
        ("n_theta", ctypes.c_uint32),
        ("n_phi", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("omega", ctypes.c_void_p),
        ("axis1", ctypes.c_void_p),
        ("axis2", ctypes.c_void_p),
        ("sin_phi", ctypes.c_void_p),
        ("cos_phi", ctypes.c_void_p),
        ("form_factor", ctypes.c_void_p),
        ("L_screen", ctypes.c_double),
    ]


# Exported symbols of include/synchrad_gb300.h (checked by the CPU tests).
class SrConfig(ctypes.Structure):
    """sr_config: work shape of the persistent mixed-precision launch."""
    _fields_ = [
        ("points_per_lane", ctypes.c_int32),
        ("lanes_per_direction", ctypes.c_int32),
        ("steps_per_stage", ctypes.c_int32),
        ("track_subsets", ctypes.c_int32),
        ("ctas", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("ms", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


EXPORTS = (
    "sr_spectrum", "sr_workspace_bytes", "sr_workspace_status", "sr_last_error",
    "sr_version", "sr_far_total", "sr_far_cartesian_comps",
    "sr_far_cartesian_comps_complex", "sr_far_spheric_comps",
    "sr_far_spheric_comps_complex", "sr_near_total", "sr_near_cartesian_comps",
    "sr_near_cartesian_comps_complex", "sr_timing_enable", "sr_timing_read",
    "sr_probe_fp32_peak", "sr_spectrum_noalloc", "sr_noalloc_status",
    "sr_far_total_forward_saved", "sr_far_total_forward_saved_df", "sr_far_forward_saved",
    "sr_far_backward_workspace_bytes", "sr_far_backward",
    "sr_far_total_backward_workspace_bytes", "sr_far_total_backward",
    "sr_autotune", "sr_config_get", "sr_config_set", "sr_config_clear", "sr_graph_create", "sr_graph_launch",
    "sr_graph_nodes", "sr_graph_destroy", "sr_near_total_forward_saved",
    "sr_near_total_backward_workspace_bytes", "sr_near_total_backward",
    "sr_selftest_wait_timeout", "sr_near_forward_saved", "sr_near_backward_workspace_bytes",
    "sr_near_backward",
)

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def _declare(L: ctypes.CDLL) -> None:
    vp, u32, dbl, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_double, ctypes.c_int
    L.sr_spectrum.restype = i32
    L.sr_spectrum.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32, i32,
                              ctypes.POINTER(vp), vp, ctypes.c_size_t, vp]
    L.sr_spectrum_noalloc.restype = i32
    L.sr_spectrum_noalloc.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32,
                                      ctypes.POINTER(vp), vp]
    L.sr_noalloc_status.restype = i32
    L.sr_noalloc_status.argtypes = [vp]
    L.sr_far_total_forward_saved.restype = i32
    L.sr_far_total_forward_saved.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid),
                                             vp, vp, vp, ctypes.c_size_t, vp]
    L.sr_far_forward_saved.restype = i32
    L.sr_far_forward_saved.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32, i32,
                                       ctypes.POINTER(vp), vp, vp, ctypes.c_size_t, vp]
    L.sr_far_backward_workspace_bytes.restype = ctypes.c_int64
    L.sr_far_backward_workspace_bytes.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid)]
    L.sr_far_backward.restype = i32
    L.sr_far_backward.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32,
                                  ctypes.POINTER(vp), vp, ctypes.POINTER(vp), vp, vp,
                                  ctypes.c_size_t, vp]
    L.sr_near_forward_saved.restype = i32
    L.sr_near_forward_saved.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32,
                                        ctypes.POINTER(vp), vp, vp, ctypes.c_size_t, vp]
    L.sr_near_backward_workspace_bytes.restype = ctypes.c_int64
    L.sr_near_backward_workspace_bytes.argtypes = [ctypes.POINTER(SrTracks),
                                                   ctypes.POINTER(SrGrid)]
    L.sr_near_backward.restype = i32
    L.sr_near_backward.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32,
                                   ctypes.POINTER(vp), vp, ctypes.POINTER(vp), vp, vp,
                                   ctypes.c_size_t, vp]
    L.sr_far_total_forward_saved_df.restype = i32
    L.sr_far_total_forward_saved_df.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid),
                                                vp, vp, vp, ctypes.c_size_t, vp]
    L.sr_far_total_backward_workspace_bytes.restype = ctypes.c_int64
    L.sr_far_total_backward_workspace_bytes.argtypes = [ctypes.POINTER(SrTracks),
                                                        ctypes.POINTER(SrGrid)]
    L.sr_far_total_backward.restype = i32
    L.sr_far_total_backward.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), vp, vp,
                                        ctypes.POINTER(vp), vp, vp, ctypes.c_size_t, vp]
    L.sr_autotune.restype = i32
    L.sr_autotune.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32, i32, dbl, vp,
                              ctypes.POINTER(SrConfig), ctypes.POINTER(SrConfig)]
    L.sr_config_get.restype = i32
    L.sr_config_get.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32, i32,
                                ctypes.POINTER(SrConfig)]
    L.sr_config_set.restype = i32
    L.sr_config_set.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32, i32,
                                ctypes.POINTER(SrConfig)]
    L.sr_config_clear.restype = i32
    L.sr_config_clear.argtypes = []
    L.sr_graph_create.restype = i32
    L.sr_graph_create.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32, i32,
                                  ctypes.POINTER(vp), vp, ctypes.c_size_t, ctypes.POINTER(vp)]
    L.sr_graph_launch.restype = i32
    L.sr_graph_launch.argtypes = [vp, vp]
    L.sr_graph_nodes.restype = i32
    L.sr_graph_nodes.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.sr_graph_destroy.restype = None
    L.sr_graph_destroy.argtypes = [vp]
    for kind in ("near",):
        fs = getattr(L, f"sr_{kind}_total_forward_saved")
        fs.restype = i32
        fs.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), vp, vp, vp,
                       ctypes.c_size_t, vp]
        wb = getattr(L, f"sr_{kind}_total_backward_workspace_bytes")
        wb.restype = ctypes.c_int64
        wb.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid)]
        bw = getattr(L, f"sr_{kind}_total_backward")
        bw.restype = i32
        bw.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), vp, vp,
                       ctypes.POINTER(vp), vp, vp, ctypes.c_size_t, vp]
    L.sr_selftest_wait_timeout.restype = i32
    L.sr_selftest_wait_timeout.argtypes = [ctypes.c_int64, vp, vp]
    L.sr_workspace_bytes.restype = ctypes.c_int64
    L.sr_workspace_bytes.argtypes = [ctypes.POINTER(SrTracks), ctypes.POINTER(SrGrid), i32, i32]
    L.sr_workspace_status.restype = i32
    L.sr_workspace_status.argtypes = [vp, vp]
    L.sr_last_error.restype = ctypes.c_char_p
    L.sr_last_error.argtypes = []
    L.sr_version.restype = i32
    L.sr_version.argtypes = []
    L.sr_timing_enable.restype = i32
    L.sr_timing_enable.argtypes = [i32]
    L.sr_timing_read.restype = i32
    L.sr_timing_read.argtypes = [ctypes.POINTER(dbl), ctypes.POINTER(i32)]
    L.sr_probe_fp32_peak.restype = i32
    L.sr_probe_fp32_peak.argtypes = [ctypes.POINTER(dbl), ctypes.POINTER(dbl), vp]
    track = [vp] * 6 + [dbl, u32, u32, u32]
    far_axes = [vp] * 5 + [u32, u32, u32, dbl, u32, vp]
    near_axes = [vp] * 4 + [dbl, u32, u32, u32, dbl, u32, vp]
    sigs = {
        "sr_far_total": [i32, i32] + [vp] + track + far_axes + [vp],
        "sr_far_cartesian_comps": [i32, i32] + [vp] * 3 + track + far_axes + [vp],
        "sr_far_cartesian_comps_complex": [i32, i32] + [vp] * 6 + track + far_axes + [vp, vp],
        "sr_far_spheric_comps": [i32, i32] + [vp] * 3 + track + far_axes + [vp],
        "sr_far_spheric_comps_complex": [i32, i32] + [vp] * 6 + track + far_axes + [vp, vp],
        "sr_near_total": [i32, i32] + [vp] + track + near_axes + [vp],
        "sr_near_cartesian_comps": [i32, i32] + [vp] * 3 + track + near_axes + [vp],
        "sr_near_cartesian_comps_complex": [i32, i32] + [vp] * 6 + track + near_axes + [vp, vp],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.restype = i32
        f.argtypes = args


def lib_path() -> Path:
    return _build.LIB


def lib(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the CUDA library; raises if unavailable."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _build.up_to_date():
            if not build_if_missing:
                raise RuntimeError(f"{_build.LIB} is missing or stale; run synchrad_gb300._build.build()")
            _build.build()
        L = ctypes.CDLL(str(_build.LIB))
        _declare(L)
        _lib = L
        return L


def check(rc: int) -> None:
    if rc != SR_OK:
        msg = lib().sr_last_error()
        raise SynchRadError(rc, msg.decode() if msg else "")
