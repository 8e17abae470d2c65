"""Host-side logic of ``synchrad/calc.py``, restated in numpy for the oracle.

TEST INFRASTRUCTURE ONLY (see :mod:`oracle`).  :func:`calculate_spectrum`
reproduces ``SynchRad.calculate_spectrum`` for track lists: grid construction
(``calc.py:355-451``), device axes (``calc.py:486-512``), radiation arrays and
FormFactor (``calc.py:453-484``), snapshot iterations (``calc.py:626-630``),
weight normalisation (``calc.py:241-265``), the per-track ``it_range``
rule (``calc.py:292-301``), the kernel argument list (``calc.py:306-322``) and
the device-to-host layout swap (``calc.py:573-577``), with one CPU kernel call
per track in place of the OpenCL launch.
"""
from __future__ import annotations

import numpy as np

from . import run_track

VEC_COMPS = {
    "cartesian": ["x", "y", "z"],
    "cartesian_complex": ["xre", "xim", "yre", "yim", "zre", "zim"],
    "spheric": ["r", "theta", "phi"],
    "spheric_complex": ["rre", "rim", "thetare", "thetaim", "phire", "phiim"],
    "total": ["total"],
}


def np_dtype(name: str):
    return {"double": np.double, "float": np.single}[name]


def init_args(args: dict) -> dict:
    """Grid construction of calc.py:355-451 (returns a new dict)."""
    a = dict(args)
    a.setdefault("mode", "far")
    a.setdefault("dtype", "double")
    dt = np_dtype(a["dtype"])
    a.setdefault("ctx", None)
    a["gridNodeNums"] = a["grid"][-1]
    a["numGridNodes"] = int(np.prod(a["gridNodeNums"]))
    No = a["gridNodeNums"][0]
    w_min, w_max = a["grid"][0]
    a.setdefault("Features", [])
    omega = np.r_[w_min:w_max:No * 1j]
    for feature in a["Features"]:
        if feature == "wavelengthGrid":
            a["wavelengths"] = np.r_[1.0 / w_max:1.0 / w_min:No * 1j]
            omega = 1.0 / a["wavelengths"]
            break
        elif feature == "logGrid":
            d_log_w = np.log(w_max / w_min) / (No - 1.0)
            omega = w_min * np.exp(d_log_w * np.arange(No))
            break
    a["omega"] = omega.astype(dt)
    a["dw"] = np.abs(omega[1:] - omega[:-1]) if No > 1 else np.array([1.0], dtype=dt)
    if a["mode"] == "far":
        Nt, Np = a["gridNodeNums"][1:]
        t0, t1 = a["grid"][1]
        p0, p1 = a["grid"][2]
        theta = np.r_[t0:t1:Nt * 1j]
        phi = p0 + (p1 - p0) / Np * np.arange(Np)
        a["dth"] = theta[1] - theta[0] if Nt > 1 else dt(1.0)
        a["dph"] = phi[1] - phi[0] if Np > 1 else dt(1.0)
        a["theta"] = theta.astype(dt)
        a["phi"] = phi.astype(dt)
        a["dV"] = a["dw"] * a["dth"] * a["dph"]
    else:
        Nr, Np = a["gridNodeNums"][1:]
        r0, r1 = a["grid"][1]
        p0, p1 = a["grid"][2]
        radius = np.r_[r0:r1:Nr * 1j]
        phi = p0 + (p1 - p0) / Np * np.arange(Np)
        a["dr"] = radius[1] - radius[0] if Nr > 1 else 1.0
        a["dph"] = phi[1] - phi[0] if Np > 1 else 1.0
        a["phi"] = phi.astype(dt)
        a["radius"] = radius.astype(dt)
        a["dV"] = a["dw"] * a["dr"] * a["dph"]
    return a


def device_axes(a: dict):
    """The arrays uploaded by calc.py:486-512, in the kernels' argument order."""
    dt = np_dtype(a["dtype"])
    om = dt(2 * np.pi) * a["omega"]
    if a["mode"] == "far":
        return [np.ascontiguousarray(v) for v in (
            om, np.sin(a["theta"]), np.cos(a["theta"]),
            np.sin(a["phi"]), np.cos(a["phi"]))]
    return [np.ascontiguousarray(v) for v in (
        om, a["radius"], np.sin(a["phi"]), np.cos(a["phi"]))]


def snap_iterations(it_range, n_snaps) -> np.ndarray:
    """calc.py:626-630."""
    return np.ascontiguousarray(
        np.linspace(*(tuple(it_range) + (int(n_snaps) + 1,)), dtype=np.uint32)[1:])


def form_factor(a: dict, sigma_particle) -> np.ndarray:
    """calc.py:475-480."""
    dt = np_dtype(a["dtype"])
    sig = dt(sigma_particle)
    exp_factor = dt(-0.5) * (dt(2 * np.pi) * a["omega"] * sig) ** 2
    return np.exp(exp_factor)


def normalise_weights(tracks, weights_normalize):
    """calc.py:241-263 (mutates the track lists in place, as the reference does)."""
    if weights_normalize in ("mean", "max"):
        weights = [t[6] for t in tracks]
        norm = np.mean(weights) if weights_normalize == "mean" else np.max(weights)
        for t in tracks:
            t[6] /= norm
    elif weights_normalize == "ones":
        for t in tracks:
            t[6] = 1.0


def calculate_spectrum(args: dict, particle_tracks, timeStep, comp="total",
                       L_screen=None, Np_max=None, it_range=None, nSnaps=1,
                       sigma_particle=0, weights_normalize=None, kind="port",
                       nthreads=None):
    """Oracle of ``SynchRad(args).calculate_spectrum(particle_tracks, ...)``.

    Returns ``(radiation, total_weight, snap_iterations, args)`` where
    ``radiation`` maps the reference's keys to float64 arrays of host layout
    ``(nSnaps, nOmega, nTheta|nR, nPhi)``.
    """
    a = init_args(args)
    dt = np_dtype(a["dtype"])
    nSnaps = np.uint32(nSnaps)
    shape = (int(nSnaps),) + tuple(a["gridNodeNums"][::-1])
    spectra = [np.zeros(shape, dtype=dt) for _ in VEC_COMPS[comp]]
    ff = form_factor(a, sigma_particle)
    axes = device_axes(a)
    step = dt(timeStep)
    snaps_global = None if it_range is None else snap_iterations(tuple(it_range), nSnaps)
    Np = len(particle_tracks)
    if Np_max is not None:
        Np = min(Np_max, Np)
    tracks = particle_tracks[:Np]
    normalise_weights(tracks, weights_normalize)
    total_weight = 0.0
    snaps = snaps_global
    for tr in tracks:
        total_weight += tr[6]
        x, y, z, ux, uy, uz = (np.ascontiguousarray(np.asarray(v).astype(dt)) for v in tr[:6])
        wp = dt(tr[6])
        it_start = np.uint32(tr[7] if len(tr) == 8 else 0)
        if it_range is None:
            it_start = np.uint32(0)
            rng = (0, x.size)
            snaps = snap_iterations(rng, nSnaps)
        else:
            rng = tuple(it_range)
        run_track(kind, a["mode"], comp, spectra, [x, y, z, ux, uy, uz], wp,
                  it_start, np.uint32(rng[-1]), np.uint32(x.size), axes,
                  a["gridNodeNums"], step, snaps, form_factor=ff,
                  L_screen=dt(L_screen) if a["mode"] == "near" else 0.0,
                  nthreads=nthreads)
    radiation = {}
    for key, arr in zip(VEC_COMPS[comp], spectra):
        radiation[key] = np.ascontiguousarray(arr.swapaxes(-1, -3), dtype=np.double)
    return radiation, total_weight, snaps, a
