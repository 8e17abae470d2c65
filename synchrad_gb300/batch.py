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


_ALIGN = 256  # every array of a packed batch starts on a 256-byte boundary


def _round_up(n: int) -> int:
    return (n + _ALIGN - 1) // _ALIGN * _ALIGN


@dataclass
class _Packing:
    """Host-side description of a batch: per-track scalars and the byte
    layout of its single contiguous buffer (CSR offsets, x..uz, weight,
    it_start, it_end, snapshot rows, in that order)."""
    lengths: np.ndarray
    offsets: np.ndarray
    weight: np.ndarray
    it_start: np.ndarray
    it_end: np.ndarray
    snaps: np.ndarray
    stride: int
    itemsize: int
    starts: list
    nbytes: int

    @property
    def total(self) -> int:
        return int(self.offsets[-1])

    @property
    def payload_bytes(self) -> int:
        return int(self.offsets.nbytes + 6 * self.total * self.itemsize + self.weight.nbytes
                   + self.it_start.nbytes + self.it_end.nbytes + self.snaps.nbytes)


def _plan(tracks, np_dtype, n_snaps, it_range) -> _Packing:
    """Per-track launch scalars of ``synchrad/calc.py:292-301, 306-307``:
    without ``it_range`` every track starts at 0 with itEnd = its length and its
    own snapshot row; with ``it_range`` the track's ``it_start`` is kept and
    every track shares one snapshot row and itEnd = it_range[-1]."""
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
    weight = np.array([float(t[6]) for t in tracks], dtype=np.float64)
    if it_range is None:
        it_start = np.zeros(n, dtype=np.uint32)
        it_end = lengths.astype(np.uint32)
        # every track's own row, snap_iterations((0, length), n_snaps), at once
        rows = np.linspace(np.zeros(n), lengths.astype(np.float64), int(n_snaps) + 1, axis=1,
                           dtype=np.uint32)[:, 1:]
        snaps = np.ascontiguousarray(rows).ravel()
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
    itemsize = np.dtype(np_dtype).itemsize
    total = int(offsets[-1])
    sizes = [offsets.nbytes] + [total * itemsize] * 6 + [weight.nbytes, 4 * n, 4 * n,
                                                        4 * snaps.size]
    starts, pos = [], 0
    for sz in sizes:
        starts.append(pos)
        pos += _round_up(sz)
    return _Packing(lengths, offsets, weight, it_start, it_end,
                    np.ascontiguousarray(snaps, dtype=np.uint32), stride, itemsize, starts,
                    max(pos, _ALIGN))


def _fill(buf: np.ndarray, pk: _Packing, tracks, np_dtype) -> None:
    """Write the batch into the uint8 host buffer ``buf`` (pk.nbytes long)."""
    def view(i, dtype, count):
        return buf[pk.starts[i]:pk.starts[i] + count * np.dtype(dtype).itemsize].view(dtype)

    n, total = len(tracks), pk.total
    view(0, np.int64, n + 1)[:] = pk.offsets
    for k in range(6):
        if n:
            np.concatenate([np.asarray(t[k]).ravel() for t in tracks],
                           out=view(1 + k, np_dtype, total))
    view(7, np.float64, n)[:] = pk.weight
    view(8, np.uint32, n)[:] = pk.it_start
    view(9, np.uint32, n)[:] = pk.it_end
    view(10, np.uint32, pk.snaps.size)[:] = pk.snaps


def _batch_on(dev: torch.Tensor, pk: _Packing, np_dtype, n_snaps, dt) -> TrackBatch:
    """TrackBatch whose arrays are views of the device buffer ``dev``."""
    tdt = torch.float32 if np_dtype == np.float32 else torch.float64
    n, total = len(pk.weight), pk.total

    def view(i, dtype, count, nbytes):
        return dev[pk.starts[i]:pk.starts[i] + count * nbytes].view(dtype)

    coords = [view(1 + k, tdt, total, pk.itemsize) for k in range(6)]
    return TrackBatch(n, tdt, total, view(0, torch.int64, n + 1, 8), coords,
                      view(7, torch.float64, n, 8), view(8, torch.int32, n, 4),
                      view(9, torch.int32, n, 4), view(10, torch.int32, pk.snaps.size, 4),
                      pk.stride, int(n_snaps), float(dt), pk.payload_bytes)


def pack_tracks(tracks, np_dtype, n_snaps, dt, it_range=None, device=None,
                pinned=True) -> TrackBatch:
    """Pack reference-format tracks ``[x, y, z, ux, uy, uz, w(, it_start)]``
    into one contiguous (pinned) host buffer and copy it to the device at once.

    Per-track launch scalars follow ``synchrad/calc.py:292-301, 306-307``
    (see ``_plan``)."""
    device = torch.device(device) if device is not None else torch.device("cuda")
    pk = _plan(tracks, np_dtype, n_snaps, it_range)
    pin = pinned and device.type == "cuda"
    host = torch.empty(pk.nbytes, dtype=torch.uint8, pin_memory=pin)
    _fill(host.numpy(), pk, tracks, np_dtype)
    dev = host.to(device, non_blocking=pin)
    return _batch_on(dev, pk, np_dtype, n_snaps, dt)


def plan_chunks(lengths, itemsize: int, min_bytes: int = 32 << 20, n_chunks: int = 8,
                lead_fraction: float = 1.0 / 32) -> list:
    """Track ranges [t0, t1) for streaming a batch to the device in pieces.

    Batches under ``min_bytes`` of coordinates stay whole.  Otherwise a small
    leading chunk (about ``lead_fraction`` of the steps: the only upload not
    hidden behind compute) is followed by about ``n_chunks`` chunks of equal
    step counts; chunks hold whole tracks."""
    lengths = np.asarray(lengths, dtype=np.int64)
    n = lengths.size
    total = int(lengths.sum())
    if n <= 1 or 6 * total * itemsize < min_bytes:
        return [(0, n)]
    cum = np.cumsum(lengths)
    cuts = [0]
    lead = max(1, int(np.searchsorted(cum, lead_fraction * total, side="left")) + 1)
    if lead < n:
        cuts.append(lead)
    rest0 = int(cum[cuts[-1] - 1])
    step = (total - rest0) / n_chunks
    for k in range(1, n_chunks):
        t = int(np.searchsorted(cum, rest0 + k * step, side="left")) + 1
        if cuts[-1] < t < n:
            cuts.append(t)
    cuts.append(n)
    return list(zip(cuts[:-1], cuts[1:]))


class TrackStream:
    """Streams a batch to the device chunk by chunk so that the host packing
    and the host-to-device copy of chunk k+1 run while chunk k is evaluated.

    Each chunk is packed into a pinned host buffer, copied on a private copy
    stream into a device buffer allocated on that stream (and marked as used
    by the chunk's compute stream), and the compute stream waits for the
    copy's event before the chunk's ``sr_spectrum`` call.  With two compute
    streams, consecutive chunks' persistent launches overlap: the next chunk's
    CTAs take the SMs the previous chunk's last work items free.  The
    reference launches one kernel per track (``synchrad/calc.py:257-267``);
    for a fixed chunking the result here is deterministic."""

    def __init__(self, device):
        self.device = torch.device(device)
        self.copy_stream = torch.cuda.Stream(self.device)

    def chunks(self, tracks, np_dtype, n_snaps, dt, it_range=None, compute_stream=None,
               plan=None, compute_streams=None):
        """Yields (TrackBatch, first track index, stream) per chunk; the batch's
        arrays are ready for work queued on that stream after the yield.
        Chunk i goes to ``compute_streams[i % len(compute_streams)]`` (default:
        ``compute_stream``, else the current stream)."""
        if compute_streams is None:
            compute_streams = [compute_stream or torch.cuda.current_stream(self.device)]
        lengths = [np.asarray(t[0]).size for t in tracks]
        if plan is None:
            plan = plan_chunks(lengths, np.dtype(np_dtype).itemsize)
        for i, (t0, t1) in enumerate(plan):
            cur = compute_streams[i % len(compute_streams)]
            part = tracks[t0:t1]
            pk = _plan(part, np_dtype, n_snaps, it_range)
            host = torch.empty(pk.nbytes, dtype=torch.uint8, pin_memory=True)
            _fill(host.numpy(), pk, part, np_dtype)
            with torch.cuda.stream(self.copy_stream):
                dev = torch.empty(pk.nbytes, dtype=torch.uint8, device=self.device)
                dev.copy_(host, non_blocking=True)
                ready = torch.cuda.Event()
                ready.record(self.copy_stream)
            dev.record_stream(cur)
            cur.wait_event(ready)
            yield _batch_on(dev, pk, np_dtype, n_snaps, dt), t0, cur


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
    if dtype_name == "double-float":
        return _lib.SR_PREC_DF
    raise ValueError(f"unknown dtype {dtype_name!r} "
                     "(expected 'double', 'float', 'mixed' or 'double-float')")


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
