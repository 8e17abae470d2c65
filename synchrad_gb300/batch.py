"""Device-side batches of tracks and grids, and the call into the CUDA library.

This replaces the per-track loop of ``SynchRad.calculate_spectrum``
(``synchrad/calc.py:257-267``: six blocking uploads and one kernel launch per
track) with one CSR upload of every track and one ``sr_spectrum`` call.
PyTorch only provides device memory and the stream; the arithmetic is in
``libsynchrad_gb300.so``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

_F64, _F32 = _lib.SR_DTYPE_F64, _lib.SR_DTYPE_F32


def snap_iterations(it_range, n_snaps) -> np.ndarray:
    """Snapshot iterations, synchrad/calc.py:626-630."""
    return np.ascontiguousarray(
        np.linspace(*(tuple(it_range) + (int(n_snaps) + 1,)), dtype=np.uint32)[1:])


@dataclass
class TrackBatch:
    """Tracks in CSR form on the device (layout of ``sr_tracks``)."""
    n_tracks: int
    dtype: torch.dtype
    total_steps: int
    offsets: torch.Tensor       # int64 [n+1]
    coords: list                # x, y, z, ux, uy, uz: [total_steps]
    weight: torch.Tensor        # float64 [n]
    it_start: torch.Tensor      # int32 (uint32 bits) [n]
    it_end: torch.Tensor        # int32 (uint32 bits) [n]
    snap_its: torch.Tensor      # int32 (uint32 bits)
    snap_stride: int
    n_snaps: int
    dt: float
    h2d_bytes: int = 0

    def c_struct(self) -> _lib.SrTracks:
        s = _lib.SrTracks()
        s.n_tracks = self.n_tracks
        s.dtype = _F32 if self.dtype == torch.float32 else _F64
        s.total_steps = self.total_steps
        s.offsets = self.offsets.data_ptr()
        s.x, s.y, s.z, s.ux, s.uy, s.uz = (c.data_ptr() for c in self.coords)
        s.weight = self.weight.data_ptr()
        s.it_start = self.it_start.data_ptr()
        s.it_end = self.it_end.data_ptr()
        s.snap_its = self.snap_its.data_ptr()
        s.snap_stride = self.snap_stride
        s.n_snaps = self.n_snaps
        s.dt = float(self.dt)
        return s


def _to_device(arr: np.ndarray, device, pinned: bool) -> torch.Tensor:
    t = torch.from_numpy(np.ascontiguousarray(arr))
    if pinned and device.type == "cuda":
        t = t.pin_memory()
    return t.to(device, non_blocking=pinned)


def _u32_view(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)


def pack_tracks(tracks, np_dtype, n_snaps, dt, it_range=None, device=None,
                pinned=True) -> TrackBatch:
    """Pack reference-format tracks ``[x, y, z, ux, uy, uz, w(, it_start)]``.

    Per-track launch scalars follow ``synchrad/calc.py:292-301, 306-307``:
    without ``it_range`` every track starts at 0 with itEnd = its length and its
    own snapshot row; with ``it_range`` the track's ``it_start`` is kept and
    every track shares one snapshot row and itEnd = it_range[-1].
    """
    device = torch.device(device) if device is not None else torch.device("cuda")
    n = len(tracks)
    lengths = np.array([np.asarray(t[0]).size for t in tracks], dtype=np.int64)
    for i, t in enumerate(tracks):
        for a in t[:6]:
            if np.asarray(a).size != lengths[i]:
                raise ValueError(f"track {i}: coordinate arrays differ in length")
    if n and lengths.min() < 1:
        raise ValueError("a track with no steps cannot be processed "
                         "(the reference's unsigned loop bounds would wrap)")
    offsets = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    total = int(offsets[-1])
    coords = []
    for k in range(6):
        buf = np.empty(total, dtype=np_dtype)
        for i, t in enumerate(tracks):
            buf[offsets[i]:offsets[i + 1]] = np.asarray(t[k])
        coords.append(buf)
    weight = np.array([float(t[6]) for t in tracks], dtype=np.float64)
    if it_range is None:
        it_start = np.zeros(n, dtype=np.uint32)
        it_end = lengths.astype(np.uint32)
        rows = [snap_iterations((0, int(L)), n_snaps) for L in lengths]
        snaps = np.concatenate(rows) if rows else np.zeros(0, np.uint32)
        stride = int(n_snaps)
    else:
        it_start = np.array([int(t[7]) if len(t) == 8 else 0 for t in tracks], dtype=np.uint32)
        end = int(it_range[-1])
        if end < 1:
            raise ValueError("it_range end must be >= 1")
        it_end = np.full(n, end, dtype=np.uint32)
        snaps = snap_iterations(tuple(it_range), n_snaps)
        stride = 0
    if n_snaps and snaps.size == 0:
        snaps = np.zeros(max(int(n_snaps), 1), np.uint32)
    host = [offsets, *coords, weight, _u32_view(it_start), _u32_view(it_end), _u32_view(snaps)]
    dev = [_to_device(a, device, pinned) for a in host]
    h2d = int(sum(a.nbytes for a in host))
    return TrackBatch(n, torch.float32 if np_dtype == np.float32 else torch.float64, total,
                      dev[0], dev[1:7], dev[7], dev[8], dev[9], dev[10], stride,
                      int(n_snaps), float(dt), h2d)


@dataclass
class GridDevice:
    """The device axes of ``synchrad/calc.py:486-512`` (omega already x 2*pi)."""
    mode: str
    dtype: torch.dtype
    n: tuple
    omega: torch.Tensor
    axis1: torch.Tensor
    axis2: torch.Tensor | None
    sin_phi: torch.Tensor
    cos_phi: torch.Tensor
    form_factor: torch.Tensor | None = None
    L_screen: float = 0.0

    def c_struct(self) -> _lib.SrGrid:
        g = _lib.SrGrid()
        g.mode = _lib.SR_MODE_FAR if self.mode == "far" else _lib.SR_MODE_NEAR
        g.dtype = _F32 if self.dtype == torch.float32 else _F64
        g.n_omega, g.n_theta, g.n_phi = (int(v) for v in self.n)
        g.omega = self.omega.data_ptr()
        g.axis1 = self.axis1.data_ptr()
        g.axis2 = self.axis2.data_ptr() if self.axis2 is not None else None
        g.sin_phi = self.sin_phi.data_ptr()
        g.cos_phi = self.cos_phi.data_ptr()
        g.form_factor = self.form_factor.data_ptr() if self.form_factor is not None else None
        g.L_screen = float(self.L_screen)
        return g


def make_grid(mode, host_axes, n, dtype, device, form_factor=None, L_screen=0.0) -> GridDevice:
    """host_axes: far (omega2pi, sinT, cosT, sinP, cosP), near (omega2pi, R, sinP, cosP)."""
    tdev = [torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in host_axes]
    ff = (torch.from_numpy(np.ascontiguousarray(form_factor)).to(device)
          if form_factor is not None else None)
    tdt = torch.float32 if np.asarray(host_axes[0]).dtype == np.float32 else torch.float64
    if mode == "far":
        return GridDevice("far", tdt, tuple(n), tdev[0], tdev[1], tdev[2], tdev[3], tdev[4],
                          ff, 0.0)
    return GridDevice("near", tdt, tuple(n), tdev[0], tdev[1], None, tdev[2], tdev[3], ff,
                      float(L_screen))


def precision_id(dtype_name: str, native: bool) -> int:
    if dtype_name == "double":
        return _lib.SR_PREC_DOUBLE
    if dtype_name == "float":
        return _lib.SR_PREC_FLOAT_NATIVE if native else _lib.SR_PREC_FLOAT
    if dtype_name == "mixed":
        return _lib.SR_PREC_MIXED
    raise ValueError(f"unknown dtype {dtype_name!r} (expected 'double', 'float' or 'mixed')")


class Workspace:
    """Grow-only device scratch buffer for ``sr_spectrum`` (256-byte aligned)."""

    def __init__(self, device):
        self.device = torch.device(device)
        self.buf: torch.Tensor | None = None

    def get(self, nbytes: int) -> torch.Tensor | None:
        if nbytes <= 0:
            return None
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(int(nbytes), dtype=torch.uint8, device=self.device)
        return self.buf


def run_spectrum(batch: TrackBatch, grid: GridDevice, comp: str, precision: int,
                 outputs: list, workspace: Workspace | None = None, stream=None,
                 check_status: bool = False) -> None:
    """Accumulate the batch's spectrum into ``outputs`` (device layout tensors)."""
    L = _lib.lib()
    cid = _lib.COMP_IDS[comp]
    if len(outputs) != _lib.N_OUT[cid]:
        raise ValueError(f"comp {comp!r} needs {_lib.N_OUT[cid]} output arrays")
    ts, gs = batch.c_struct(), grid.c_struct()
    need = L.sr_workspace_bytes(ctypes.byref(ts), ctypes.byref(gs), cid, precision)
    if need < 0:
        _lib.check(_lib.SR_ERR_INVALID if need == -1 else int(need))
    ws = (workspace or Workspace(outputs[0].device)).get(int(need))
    outs = (ctypes.c_void_p * 6)(*([o.data_ptr() for o in outputs] + [None] * (6 - len(outputs))))
    if stream is None:
        stream = torch.cuda.current_stream(outputs[0].device)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    rc = L.sr_spectrum(ctypes.byref(ts), ctypes.byref(gs), cid, precision, outs,
                       ws.data_ptr() if ws is not None else None,
                       ctypes.c_size_t(int(need) if ws is not None else 0), sptr)
    _lib.check(rc)
    if check_status and ws is not None:
        _lib.check(L.sr_workspace_status(ctypes.c_void_p(ws.data_ptr()), sptr))


def autotune(batch: TrackBatch, grid: GridDevice, comp: str = "total",
             precision: int = _lib.SR_PREC_MIXED, budget_ms: float = 3000.0,
             stream=None) -> dict:
    """Tune the work shape of the persistent mixed-precision launch for this
    batch's sizes (``sr_autotune``); later ``run_spectrum`` calls with the same
    sizes use the choice.  Returns {'best': ..., 'default': ...} shapes with
    their times on the tuning sample."""
    L = _lib.lib()
    ts, gs = batch.c_struct(), grid.c_struct()
    best, dflt = _lib.SrConfig(), _lib.SrConfig()
    if stream is None:
        stream = torch.cuda.current_stream(batch.offsets.device)
    _lib.check(L.sr_autotune(ctypes.byref(ts), ctypes.byref(gs), _lib.COMP_IDS[comp], precision,
                             float(budget_ms), ctypes.c_void_p(stream.cuda_stream),
                             ctypes.byref(best), ctypes.byref(dflt)))
    return {"best": best.as_dict(), "default": dflt.as_dict()}


def current_config(batch: TrackBatch, grid: GridDevice, comp: str = "total",
                   precision: int = _lib.SR_PREC_MIXED) -> dict:
    """The work shape ``run_spectrum`` uses for these sizes."""
    L = _lib.lib()
    ts, gs = batch.c_struct(), grid.c_struct()
    c = _lib.SrConfig()
    _lib.check(L.sr_config_get(ctypes.byref(ts), ctypes.byref(gs), _lib.COMP_IDS[comp],
                               precision, ctypes.byref(c)))
    return c.as_dict()


def set_config(batch: TrackBatch, grid: GridDevice, comp: str = "total",
               precision: int = _lib.SR_PREC_MIXED, points_per_lane: int = 32,
               lanes_per_direction: int = 32, steps_per_stage: int = 128,
               track_subsets: int = 0) -> None:
    """Pin a work shape for this batch's sizes (``sr_config_set``)."""
    c = _lib.SrConfig(points_per_lane, lanes_per_direction, steps_per_stage, track_subsets, 0, 0,
                      0.0)
    ts, gs = batch.c_struct(), grid.c_struct()
    _lib.check(_lib.lib().sr_config_set(ctypes.byref(ts), ctypes.byref(gs), _lib.COMP_IDS[comp],
                                        precision, ctypes.byref(c)))


class SpectrumGraph:
    """One ``sr_spectrum`` call captured as a CUDA graph (``sr_graph_create``)
    and replayed by ``launch``; the batch, grid, outputs and workspace must stay
    alive and in place while the graph is used."""

    def __init__(self, batch: TrackBatch, grid: GridDevice, comp: str, precision: int,
                 outputs: list, workspace: Workspace | None = None):
        L = _lib.lib()
        cid = _lib.COMP_IDS[comp]
        if len(outputs) != _lib.N_OUT[cid]:
            raise ValueError(f"comp {comp!r} needs {_lib.N_OUT[cid]} output arrays")
        ts, gs = batch.c_struct(), grid.c_struct()
        need = L.sr_workspace_bytes(ctypes.byref(ts), ctypes.byref(gs), cid, precision)
        if need < 0:
            _lib.check(_lib.SR_ERR_INVALID)
        self.workspace = workspace or Workspace(outputs[0].device)
        ws = self.workspace.get(int(need))
        outs = (ctypes.c_void_p * 6)(*([o.data_ptr() for o in outputs]
                                       + [None] * (6 - len(outputs))))
        h = ctypes.c_void_p()
        _lib.check(L.sr_graph_create(ctypes.byref(ts), ctypes.byref(gs), cid, precision, outs,
                                     ws.data_ptr() if ws is not None else None,
                                     ctypes.c_size_t(int(need) if ws is not None else 0),
                                     ctypes.byref(h)))
        self._keep = (batch, grid, outputs, ws)
        self.handle = h

    def launch(self, stream=None) -> None:
        if self.handle is None:
            raise RuntimeError("graph destroyed")
        if stream is None:
            stream = torch.cuda.current_stream(self._keep[2][0].device)
        _lib.check(_lib.lib().sr_graph_launch(self.handle, ctypes.c_void_p(stream.cuda_stream)))

    def nodes(self) -> tuple:
        k, n = ctypes.c_int(0), ctypes.c_int(0)
        _lib.check(_lib.lib().sr_graph_nodes(self.handle, ctypes.byref(k), ctypes.byref(n)))
        return k.value, n.value

    def close(self) -> None:
        if self.handle is not None:
            _lib.lib().sr_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
