"""Differentiable spectra: ``torch.autograd.Function`` over the hand-written
adjoint kernels.

``far_total_spectrum(x, y, z, ux, uy, uz, w, layout)`` and
``near_total_spectrum(...)`` return the mixed-precision (or, far field,
double-float: ``make_layout(precision=...)``) far-field or near-field
(screen) spectrum ``S`` (comp 'total', one snapshot, device layout
``[nPhi, nTheta|nR, nOmega]``) of a batch of tracks given as concatenated
float64 CUDA tensors (CSR order of ``layout.offsets``); the backward calls
``sr_far_total_backward`` / ``sr_near_total_backward`` and returns dL/dx ..
dL/duz (per step) and dL/dw (per track).  The |dphase| < pi mask of the
reference is held fixed (it is a step function of the coordinates).

The reference has no gradients; these extend its integrals
(``synchrad/kernel_farfield.cl:59-107``, ``synchrad/kernel_nearfield.cl:58-102``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .batch import GridDevice, TrackBatch, Workspace, make_grid, snap_iterations


@dataclass
class SpectrumLayout:
    """Everything of a batch that is not differentiated."""
    offsets: torch.Tensor        # int64 [n+1] on the device
    it_start: torch.Tensor       # int32 [n]
    it_end: torch.Tensor         # int32 [n]
    snap_its: torch.Tensor       # int32 [n][n_snaps] (each track's own snapshot row)
    dt: float
    grid: GridDevice
    workspace: Workspace
    mode: str = "far"
    precision: str = "mixed"     # forward arithmetic: 'mixed' or 'double-float' (far field)
    n_snaps: int = 1             # snapshots per track (rows of snap_its)

    @property
    def n_tracks(self) -> int:
        return int(self.offsets.numel() - 1)

    @property
    def n_points(self) -> int:
        return int(np.prod(self.grid.n))


FarLayout = SpectrumLayout


def make_layout(lengths, dt, host_axes, n, device="cuda", mode="far",
                L_screen=0.0, precision="mixed", form_factor=None,
                n_snaps=1) -> SpectrumLayout:
    """Layout for tracks of the given lengths with the reference's per-track
    rules (it_start = 0, itEnd = length, snapshot iterations
    ``linspace(0, length, n_snaps + 1)[1:]``, synchrad/calc.py:297-301, 626-630);
    with several snapshots the spectra are ``[n_snaps, ...]`` and each
    snapshot's gradient flows to the steps it accumulated.
    host_axes: far (omega2pi, sinT, cosT, sinP, cosP), near (omega2pi, R,
    sinP, cosP) as from ``synchrad/calc.py:486-512``.

    ``precision`` is the forward's arithmetic: 'mixed' (FP32 bulk, ~1e-7 of
    the spectrum) or 'double-float' (far field, FP64-class spectrum), for
    losses that amplify the spectrum's error, such as a misfit S - T that is a
    small fraction of S.  The backward is the same for both.  ``form_factor``
    (one value per omega, ``synchrad/calc.py:475-480``) is needed by the far
    'cartesian_complex' comp."""
    if precision not in ("mixed", "double-float"):
        raise ValueError(f"precision {precision!r}: 'mixed' or 'double-float'")
    if precision == "double-float" and mode != "far":
        raise ValueError("the double-float forward is far field only")
    device = torch.device(device)
    lengths = np.asarray(lengths, dtype=np.int64)
    if np.any(lengths < 1):
        raise ValueError("every track needs at least one step")
    offsets = np.zeros(lengths.size + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    if int(n_snaps) < 1:
        raise ValueError("at least one snapshot")
    snaps = np.concatenate([snap_iterations((0, int(L)), int(n_snaps)) for L in lengths])
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
    grid = make_grid(mode, host_axes, n, torch.float64, device, L_screen=L_screen,
                     form_factor=None if form_factor is None
                     else np.asarray(form_factor, dtype=np.float64))
    return SpectrumLayout(t(offsets), t(np.zeros(lengths.size, np.int32)),
                          t(lengths.astype(np.uint32).view(np.int32)),
                          t(snaps.astype(np.uint32).view(np.int32)), float(dt), grid,
                          Workspace(device), mode, precision, int(n_snaps))


def _tracks_struct(coords, w, layout: FarLayout) -> TrackBatch:
    return TrackBatch(layout.n_tracks, torch.float64, int(coords[0].numel()), layout.offsets,
                      list(coords), w, layout.it_start, layout.it_end, layout.snap_its,
                      layout.n_snaps, layout.n_snaps, layout.dt)


def _spectrum_shape(layout: SpectrumLayout) -> tuple:
    nO, nT, nP = layout.grid.n
    return (nP, nT, nO) if layout.n_snaps == 1 else (layout.n_snaps, nP, nT, nO)


_SAVED_FLOATS = {"far": 4, "near": 8}  # per point and track


class TotalSpectrum(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, z, ux, uy, uz, w, layout: SpectrumLayout):
        L = _lib.lib()
        coords = [c.detach().contiguous() for c in (x, y, z, ux, uy, uz)]
        for c in coords:
            if c.dtype != torch.float64 or not c.is_cuda:
                raise TypeError("track tensors must be float64 CUDA tensors")
        wd = w.detach().contiguous().to(torch.float64)
        batch = _tracks_struct(coords, wd, layout)
        ts, gs = batch.c_struct(), layout.grid.c_struct()
        P = layout.n_points
        spec = torch.zeros(_spectrum_shape(layout), dtype=torch.float64, device=x.device)
        saved = torch.empty(layout.n_tracks * layout.n_snaps * P * _SAVED_FLOATS[layout.mode],
                            dtype=torch.float32, device=x.device)
        df_fwd = layout.precision == "double-float"
        prec = _lib.SR_PREC_DF if df_fwd else _lib.SR_PREC_MIXED
        need = L.sr_workspace_bytes(ctypes.byref(ts), ctypes.byref(gs), 0, prec)
        if need < 0:
            _lib.check(_lib.SR_ERR_INVALID if need == -1 else int(need))
        ws = layout.workspace.get(max(int(need), 256))
        stream = ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
        fwd = getattr(L, f"sr_{layout.mode}_total_forward_saved" + ("_df" if df_fwd else ""))
        _lib.check(fwd(ctypes.byref(ts), ctypes.byref(gs), spec.data_ptr(), saved.data_ptr(),
                       ws.data_ptr(), ctypes.c_size_t(int(need)), stream))
        ctx.save_for_backward(*coords, wd, saved)
        ctx.layout = layout
        return spec

    @staticmethod
    def backward(ctx, grad_spec):
        L = _lib.lib()
        *coords, wd, saved = ctx.saved_tensors
        layout = ctx.layout
        batch = _tracks_struct(coords, wd, layout)
        ts, gs = batch.c_struct(), layout.grid.c_struct()
        g = grad_spec.detach().contiguous().to(torch.float64)
        grads = [torch.empty_like(c) for c in coords]
        gw = torch.empty(layout.n_tracks, dtype=torch.float64, device=g.device)
        need = getattr(L, f"sr_{layout.mode}_total_backward_workspace_bytes")(
            ctypes.byref(ts), ctypes.byref(gs))
        if need < 0:
            _lib.check(_lib.SR_ERR_INVALID)
        ws = layout.workspace.get(max(int(need), 256))
        ptrs = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in grads])
        stream = ctypes.c_void_p(torch.cuda.current_stream(g.device).cuda_stream)
        bwd = getattr(L, f"sr_{layout.mode}_total_backward")
        _lib.check(bwd(ctypes.byref(ts), ctypes.byref(gs), g.data_ptr(), saved.data_ptr(), ptrs,
                       gw.data_ptr(), ws.data_ptr(), ctypes.c_size_t(int(need)), stream))
        return (*grads, gw, None)


FarTotalSpectrum = TotalSpectrum


class SpectrumComps(torch.autograd.Function):
    """Every comp of the far field or the near field (the layout's mode): the
    forward returns the comp's outputs (the reference's keys in order, e.g.
    x, y, z or xre, xim, ..., zim) and the backward takes a gradient for each
    (None counts as zero)."""

    @staticmethod
    def forward(ctx, x, y, z, ux, uy, uz, w, layout: SpectrumLayout, comp: str):
        L = _lib.lib()
        cid = _lib.COMP_IDS[comp]
        coords = [c.detach().contiguous() for c in (x, y, z, ux, uy, uz)]
        for c in coords:
            if c.dtype != torch.float64 or not c.is_cuda:
                raise TypeError("track tensors must be float64 CUDA tensors")
        wd = w.detach().contiguous().to(torch.float64)
        batch = _tracks_struct(coords, wd, layout)
        ts, gs = batch.c_struct(), layout.grid.c_struct()
        P = layout.n_points
        outs = [torch.zeros(_spectrum_shape(layout), dtype=torch.float64, device=x.device)
                for _ in range(_lib.N_OUT[cid])]
        saved = torch.empty(layout.n_tracks * layout.n_snaps * P * _SAVED_FLOATS[layout.mode],
                            dtype=torch.float32, device=x.device)
        prec = _lib.SR_PREC_DF if layout.precision == "double-float" else _lib.SR_PREC_MIXED
        need = L.sr_workspace_bytes(ctypes.byref(ts), ctypes.byref(gs), cid, prec)
        if need < 0:
            _lib.check(_lib.SR_ERR_INVALID if need == -1 else int(need))
        ws = layout.workspace.get(max(int(need), 256))
        ptrs = (ctypes.c_void_p * 6)(*([o.data_ptr() for o in outs] + [None] * (6 - len(outs))))
        stream = ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
        if layout.mode == "far":
            rc = L.sr_far_forward_saved(ctypes.byref(ts), ctypes.byref(gs), cid, prec, ptrs,
                                        saved.data_ptr(), ws.data_ptr(),
                                        ctypes.c_size_t(int(need)), stream)
        else:
            rc = L.sr_near_forward_saved(ctypes.byref(ts), ctypes.byref(gs), cid, ptrs,
                                         saved.data_ptr(), ws.data_ptr(),
                                         ctypes.c_size_t(int(need)), stream)
        _lib.check(rc)
        ctx.save_for_backward(*coords, wd, saved)
        ctx.layout = layout
        ctx.comp = comp
        return tuple(outs)

    @staticmethod
    def backward(ctx, *grad_outs):
        L = _lib.lib()
        *coords, wd, saved = ctx.saved_tensors
        layout = ctx.layout
        cid = _lib.COMP_IDS[ctx.comp]
        batch = _tracks_struct(coords, wd, layout)
        ts, gs = batch.c_struct(), layout.grid.c_struct()
        dev = coords[0].device
        g = [(gr.detach().contiguous().to(torch.float64) if gr is not None
              else torch.zeros(_spectrum_shape(layout), dtype=torch.float64, device=dev))
             for gr in grad_outs]
        grads = [torch.empty_like(c) for c in coords]
        gw = torch.empty(layout.n_tracks, dtype=torch.float64, device=dev)
        need = getattr(L, f"sr_{layout.mode}_backward_workspace_bytes")(ctypes.byref(ts),
                                                                         ctypes.byref(gs))
        if need < 0:
            _lib.check(_lib.SR_ERR_INVALID)
        ws = layout.workspace.get(max(int(need), 256))
        gptrs = (ctypes.c_void_p * 6)(*([t.data_ptr() for t in g] + [None] * (6 - len(g))))
        tptrs = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in grads])
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        bwd = getattr(L, f"sr_{layout.mode}_backward")
        _lib.check(bwd(ctypes.byref(ts), ctypes.byref(gs), cid, gptrs, saved.data_ptr(), tptrs,
                       gw.data_ptr(), ws.data_ptr(), ctypes.c_size_t(int(need)), stream))
        return (*grads, gw, None, None)


def far_spectrum(x, y, z, ux, uy, uz, w, layout: SpectrumLayout, comp: str = "total"):
    """Differentiable far-field spectrum of any comp: a tuple of its outputs
    (device layout ``[nPhi, nTheta, nOmega]`` each, the reference's keys in
    order: ``synchrad/calc.py:458-465``)."""
    if layout.mode != "far":
        raise ValueError("far_spectrum needs a far-field layout")
    if comp not in _lib.COMP_IDS:
        raise ValueError(f"unknown comp {comp!r}")
    return SpectrumComps.apply(x, y, z, ux, uy, uz, w, layout, comp)


def near_spectrum(x, y, z, ux, uy, uz, w, layout: SpectrumLayout, comp: str = "total"):
    """Differentiable near-field (screen) spectrum of comp 'total', 'cartesian'
    or 'cartesian_complex': a tuple of its outputs (device layout
    ``[nPhi, nR, nOmega]`` each)."""
    if layout.mode != "near":
        raise ValueError("near_spectrum needs a near-field layout (mode='near')")
    if comp not in ("total", "cartesian", "cartesian_complex"):
        raise ValueError(f"comp {comp!r} is not a near-field comp")
    return SpectrumComps.apply(x, y, z, ux, uy, uz, w, layout, comp)


def far_total_spectrum(x, y, z, ux, uy, uz, w, layout: SpectrumLayout) -> torch.Tensor:
    """Differentiable mixed-precision far-field spectrum (see module docstring)."""
    if layout.mode != "far":
        raise ValueError("far_total_spectrum needs a far-field layout")
    return TotalSpectrum.apply(x, y, z, ux, uy, uz, w, layout)


def near_total_spectrum(x, y, z, ux, uy, uz, w, layout: SpectrumLayout) -> torch.Tensor:
    """Differentiable mixed-precision near-field (screen) spectrum."""
    if layout.mode != "near":
        raise ValueError("near_total_spectrum needs a near-field layout (mode='near')")
    return TotalSpectrum.apply(x, y, z, ux, uy, uz, w, layout)


def total_spectrum_fn(mode: str):
    """far_total_spectrum or near_total_spectrum by mode."""
    return {"far": far_total_spectrum, "near": near_total_spectrum}[mode]
