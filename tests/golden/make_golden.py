"""Generate the golden vectors in tests/golden/*.npz.

Each case is a full ``SynchRad(args).calculate_spectrum(tracks, ...)`` call
run by the reference's own host code (``ref_host_flow.py``: the body of
``synchrad/calc.py`` parsed from the reference tree) on the reference's own
kernel source compiled for the CPU (``oracle/_ref``, built by
``oracle/build_ref.sh``).  Every case is also run through the oracle's host
restatement (``oracle/host.py``) and must agree bit for bit.  The inputs
(tracks, grid, call arguments) are stored next to the outputs so the GPU
parity tests can replay them without regenerating anything.

Run from the repository root, where the reference tree is available:

    python tests/golden/make_golden.py [name-prefix ...]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle import host  # noqa: E402

sys.path.insert(0, str(Path(__file__).resolve().parent))
import ref_host_flow  # noqa: E402
from synchrad_gb300 import workloads as wl  # noqa: E402

OUT = Path(__file__).resolve().parent


def _undulator_pair(n_periods=4, spp=16, dtype=np.float64, seed=1):
    tracks, dt, k_res = wl.analytic_undulator_tracks(
        n_particles=2, n_periods=n_periods, steps_per_period=spp, seed=seed)
    out = []
    for i, t in enumerate(tracks):
        t = [np.asarray(a, dtype=dtype) for a in t[:6]] + [0.7 + 0.6 * i, 0]
        out.append(t)
    return out, dt, k_res


def cases():
    """Yield (name, args, tracks, call_kwargs)."""
    tr, dt, kres = _undulator_pair()
    far_grid = [(0.02 * kres, 1.1 * kres), (0, 2 / 100.0), (0, 2 * np.pi), (24, 6, 5)]
    sigma = 1e-5
    for dtype in ("double", "float"):
        for comp in ("total", "cartesian", "cartesian_complex", "spheric",
                     "spheric_complex"):
            tt = tr if dtype == "double" else [
                [np.asarray(a, np.float32) for a in t[:6]] + t[6:] for t in tr]
            yield (f"far_{comp}_{dtype}", {"grid": far_grid, "dtype": dtype}, tt,
                   dict(timeStep=dt, comp=comp, nSnaps=3 if comp != "total" else 1,
                        sigma_particle=sigma))
    near_grid = [(0.02 * kres, 1.1 * kres), (0, 1000 / 100.0), (0, 2 * np.pi), (20, 6, 4)]
    for dtype in ("double", "float"):
        for comp in ("total", "cartesian", "cartesian_complex"):
            tt = tr if dtype == "double" else [
                [np.asarray(a, np.float32) for a in t[:6]] + t[6:] for t in tr]
            yield (f"near_{comp}_{dtype}",
                   {"grid": near_grid, "mode": "near", "dtype": dtype}, tt,
                   dict(timeStep=dt, comp=comp, nSnaps=2, L_screen=1000.0,
                        sigma_particle=sigma))

    # global it_range with per-track it_start (8-element tracks), 4 snapshots
    t3, dt3, k3 = _undulator_pair(n_periods=3, spp=16, seed=2)
    t3 = [t3[0][:6] + [1.0, 0], t3[1][:6] + [1.3, 17]]
    yield ("far_total_itrange", {"grid": far_grid, "dtype": "double"}, t3,
           dict(timeStep=dt3, comp="total", nSnaps=4, it_range=(0, 90)))
    yield ("far_cartesian_itrange_long", {"grid": far_grid, "dtype": "double"}, t3,
           dict(timeStep=dt3, comp="cartesian", nSnaps=3, it_range=(5, 140)))

    # ragged tracks (different lengths), weights normalised by the mean
    rng = np.random.default_rng(5)
    rag = []
    for n, g in ((40, 100.0), (73, 101.0), (2, 99.0), (1, 100.0), (57, 100.5)):
        t, _, _ = _undulator_pair(n_periods=3, spp=16, seed=int(rng.integers(100)))
        rag.append([a[:n].copy() for a in t[0][:6]] + [float(rng.uniform(0.5, 2)), 0])
    yield ("far_total_ragged_wmean", {"grid": far_grid, "dtype": "double"}, rag,
           dict(timeStep=dt, comp="total", nSnaps=2, weights_normalize="mean"))

    # low-frequency grid down to ~0: the first step passes the |dphase| < pi
    # test (phasePrev starts at 0), and a coarse track trips the mask mid-track
    coarse, dtc, kc = _undulator_pair(n_periods=4, spp=3, seed=3)
    low_grid = [(0.0, 0.6 * kc), (0, 3 / 100.0), (0, 2 * np.pi), (40, 5, 4)]
    yield ("far_total_mask_lowfreq", {"grid": low_grid, "dtype": "double"}, coarse,
           dict(timeStep=dtc, comp="total", nSnaps=1))
    yield ("far_spheric_mask_lowfreq", {"grid": low_grid, "dtype": "double"}, coarse,
           dict(timeStep=dtc, comp="spheric", nSnaps=2))
    yield ("near_total_mask_lowfreq",
           {"grid": [(0.0, 0.6 * kc), (0, 30.0), (0, 2 * np.pi), (40, 5, 4)],
            "mode": "near", "dtype": "double"}, coarse,
           dict(timeStep=dtc, comp="total", nSnaps=1, L_screen=1000.0))

    # non-uniform frequency axes
    for feat in ("logGrid", "wavelengthGrid"):
        yield (f"far_total_{feat}",
               {"grid": far_grid, "dtype": "double", "Features": [feat]}, tr,
               dict(timeStep=dt, comp="total", nSnaps=1))

    # more snapshots than iterations: repeated snapshot iterations leave the
    # reference's snapshot index stuck after the first repeat
    short, dts, ks = _undulator_pair(n_periods=2, spp=8, seed=4)
    short = [[a[10:22].copy() for a in t[:6]] + [1.0, 0] for t in short]
    yield ("far_total_snaps_repeat", {"grid": far_grid, "dtype": "double"}, short,
           dict(timeStep=dts, comp="total", nSnaps=8, it_range=(2, 8)))
    # a first snapshot at iteration 1 can never fire (it_glob + 2 >= 2): all zero
    yield ("far_total_snaps_stuck", {"grid": far_grid, "dtype": "double"}, short,
           dict(timeStep=dts, comp="total", nSnaps=9))

    # the near field through the same host rules: it_range with per-track
    # it_start and 4 snapshots, ragged tracks with mean-normalised weights, a
    # log-spaced omega axis, repeated snapshot iterations
    near_args = {"grid": near_grid, "mode": "near", "dtype": "double"}
    yield ("near_total_itrange", near_args, t3,
           dict(timeStep=dt3, comp="total", nSnaps=4, it_range=(0, 90), L_screen=1000.0))
    yield ("near_total_ragged_wmean", near_args, rag,
           dict(timeStep=dt, comp="total", nSnaps=2, weights_normalize="mean", L_screen=1000.0))
    yield ("near_total_logGrid", dict(near_args, Features=["logGrid"]), tr,
           dict(timeStep=dt, comp="total", nSnaps=1, L_screen=1000.0))
    yield ("near_cartesian_snaps_repeat", near_args, short,
           dict(timeStep=dts, comp="cartesian", nSnaps=8, it_range=(2, 8), L_screen=1000.0))


def main(only=()):
    """Write every case, or only those whose names start with one of `only`."""
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref is not buildable here (reference tree missing)")
    manifest = {}
    for name, args, tracks, kw in cases():
        if only and not any(name.startswith(o) for o in only):
            continue
        call = dict(kw)
        rad, tw, snaps, a = ref_host_flow.calculate_spectrum(
            dict(args), [list(t) for t in tracks], **call)
        o_rad, o_tw, o_snaps, _ = host.calculate_spectrum(
            dict(args), [list(t) for t in tracks], kind="ref", nthreads=4, **call)
        assert sorted(o_rad) == sorted(rad) and o_tw == tw, name
        assert np.array_equal(np.asarray(o_snaps), np.asarray(snaps)), name
        for key in rad:
            assert np.array_equal(o_rad[key], rad[key]), (name, key)
        data = {}
        for i, t in enumerate(tracks):
            for j, key in enumerate(("x", "y", "z", "ux", "uy", "uz")):
                data[f"track{i}_{key}"] = np.asarray(t[j])
            data[f"track{i}_meta"] = np.array(
                [float(t[6]), float(t[7]) if len(t) == 8 else -1.0])
        for key, arr in rad.items():
            data[f"out_{key}"] = arr
        # the omega axis the reference was evaluated on: a log-spaced axis
        # comes from np.exp, whose last bit depends on the platform, and a
        # near-field phase of ~1e8 rad turns one ulp of omega into ~1e-8 rad
        data["omega"] = np.asarray(a["omega"])
        data["total_weight"] = np.array(float(tw))
        data["snap_iterations"] = np.asarray(snaps)
        meta = {"args": {k: (list(map(list, v[:-1])) + [list(v[-1])] if k == "grid" else v)
                         for k, v in args.items()},
                "call": {k: (list(v) if isinstance(v, tuple) else v) for k, v in call.items()},
                "n_tracks": len(tracks)}
        data["meta_json"] = np.array(json.dumps(meta))
        np.savez_compressed(OUT / f"{name}.npz", **data)
        manifest[name] = {k: float(np.abs(v).max()) for k, v in rad.items()}
        print(f"{name}: " + ", ".join(f"{k}={v:.3e}" for k, v in manifest[name].items()))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
