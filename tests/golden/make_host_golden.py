"""Golden vectors of the reference's host-side Python: grid construction
(``SynchRad._init_args``, synchrad/calc.py:355-451), result arrays and
FormFactor (``_init_raditaion``, :453-484), device axes (``_init_data``,
:486-512), snapshot iterations (``_set_snap_iterations``, :626-630) and the
``Utilities`` post-processing (synchrad/utils.py:21-166), and the HDF5
layout ``calculate_spectrum`` writes (synchrad/calc.py:274-290), recorded
through ``tests/fake_h5py.py`` while the reference's host flow
(``ref_host_flow.py``) runs on its CPU-built kernels.

The reference package cannot be imported here (it needs pyopencl, mako and
h5py), so this script runs the reference's own function bodies: it parses
synchrad/calc.py and synchrad/utils.py from the reference tree, keeps the
functions above (and utils.py's module-level constants), drops the imports of
the missing packages, and executes them with numpy and scipy; the OpenCL
array module is replaced by numpy (``to_device`` returns its host array,
``zeros`` a numpy array of the same shape and dtype).  numpy 2.x has
no ``np.trapz``; it is supplied as ``np.trapezoid`` (the same function under
its new name).  Inputs and outputs go to ``tests/golden/host_golden.npz``.

Run from the repository root, where the reference tree is available:

    python tests/golden/make_host_golden.py
"""
from __future__ import annotations

import ast
import os
import json
import sys
import types
from pathlib import Path

import numpy as np

REF = Path(os.environ.get("SR_REFERENCE_ROOT", "/root/reference")) / "synchrad"
OUT = Path(__file__).resolve().parent / "host_golden.npz"


def _numpy_with_trapz():
    shim = types.ModuleType("numpy")
    shim.__dict__.update(np.__dict__)
    if not hasattr(np, "trapz"):
        shim.trapz = np.trapezoid
    return shim


class _HostArrays:
    """Stand-in for pyopencl.array: the arrays stay on the host."""

    @staticmethod
    def to_device(queue, a):
        return np.array(a)

    @staticmethod
    def zeros(queue, shape, dtype):
        return np.zeros(shape, dtype=dtype)


def load_calc_functions():
    """The reference's SynchRad host methods as methods of a bare class (the
    device upload at the end of _set_snap_iterations removed)."""
    src = (REF / "calc.py").read_text()
    tree = ast.parse(src)
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "SynchRad")
    funcs = [n for n in cls.body
             if isinstance(n, ast.FunctionDef) and n.name in (
                 "_init_args", "_set_snap_iterations", "_init_data", "_init_raditaion")]
    for f in funcs:
        if f.name == "_set_snap_iterations":
            # keep the host computation, drop `arrcl.to_device(self.queue, ...)`
            f.body = [s for s in f.body if "arrcl" not in ast.unparse(s)]
    kw = {"type_params": []} if "type_params" in ast.ClassDef._fields else {}
    mod = ast.Module(body=[ast.ClassDef(name="RefCalc", bases=[], keywords=[], body=funcs,
                                        decorator_list=[], **kw)], type_ignores=[])
    ast.fix_missing_locations(mod)
    ns = {"np": _numpy_with_trapz(), "arrcl": _HostArrays}
    exec(compile(mod, str(REF / "calc.py"), "exec"), ns)
    return ns["RefCalc"]


def load_utilities():
    """The reference's Utilities class and constants, imports of h5py, tvtk and
    the converters module left out (none of them is used by the methods run)."""
    src = (REF / "utils.py").read_text()
    tree = ast.parse(src)
    body = []
    for n in tree.body:
        if isinstance(n, (ast.Import, ast.ImportFrom, ast.Try)):
            continue
        body.append(n)
    mod = ast.Module(body=body, type_ignores=[])
    from scipy.constants import alpha, c, e, epsilon_0, hbar, m_e
    from scipy.interpolate import griddata
    from scipy.ndimage import gaussian_filter
    ns = {"np": _numpy_with_trapz(), "m_e": m_e, "c": c, "e": e, "epsilon_0": epsilon_0,
          "hbar": hbar, "alpha_fs": alpha, "griddata": griddata,
          "gaussian_filter": gaussian_filter, "tvtk_installed": False}
    exec(compile(mod, str(REF / "utils.py"), "exec"), ns)
    return ns["Utilities"]


GRID_CASES = {
    "far_double": {"grid": [(100.0, 2000.0), (0.0, 0.02), (0.0, 2 * np.pi), (16, 8, 6)],
                   "dtype": "double"},
    "far_float": {"grid": [(100.0, 2000.0), (0.0, 0.02), (0.0, 2 * np.pi), (16, 8, 6)],
                  "dtype": "float"},
    "far_log": {"grid": [(100.0, 20000.0), (0.0, 0.02), (0.0, 2 * np.pi), (24, 5, 4)],
                "dtype": "double", "Features": ["logGrid"]},
    "far_wavelength": {"grid": [(100.0, 20000.0), (0.0, 0.02), (0.0, np.pi), (24, 5, 4)],
                       "dtype": "double", "Features": ["wavelengthGrid"]},
    "far_single_nodes": {"grid": [(500.0, 500.0), (0.01, 0.01), (0.0, 2 * np.pi), (1, 1, 1)],
                         "dtype": "double"},
    "near_double": {"grid": [(100.0, 2000.0), (0.0, 10.0), (0.0, 2 * np.pi), (16, 7, 6)],
                    "mode": "near", "dtype": "double"},
    "near_float_log": {"grid": [(100.0, 2000.0), (1.0, 10.0), (0.0, 2 * np.pi), (12, 5, 3)],
                       "mode": "near", "dtype": "float", "Features": ["logGrid"]},
}
GRID_KEYS = ("omega", "wavelengths", "dw", "theta", "phi", "radius", "dth", "dph", "dr", "dV",
             "numGridNodes")
# (grid case, comp, nSnaps, sigma_particle, L_screen)
RADIATION_CASES = [("far_double", "total", 1, 0.0, None),
                   ("far_double", "cartesian_complex", 3, 1e-4, None),
                   ("far_float", "spheric_complex", 2, 2e-5, None),
                   ("far_log", "spheric", 1, 0.0, None),
                   ("near_double", "cartesian", 2, 1e-4, 1000.0),
                   ("near_float_log", "cartesian_complex", 1, 3e-5, 250.0)]
SNAP_CASES = [((0, 100), 1), ((0, 100), 4), ((5, 140), 3), ((2, 8), 8), ((0, 7), 9),
              ((0, 1), 1), ((10, 10), 2), ((0, 4000), 7)]


def ref_args(RefCalc, args):
    obj = RefCalc()
    a = json.loads(json.dumps(args))  # fresh lists; 'is' string tests see interned literals
    a["grid"] = [tuple(v) for v in a["grid"]]
    for key in ("dtype", "mode"):
        if key in a:
            a[key] = {"double": "double", "float": "float", "far": "far", "near": "near"}[a[key]]
    obj._init_args(a)
    return obj


# (grid case, calculate_spectrum arguments) of the HDF5-layout cases; a
# "file_tracks" entry names a track file written by write_track_file
H5_CASES = [
    ("far_double", {"comp": "cartesian", "nSnaps": 2, "it_range": [0, 60],
                    "sigma_particle": 1e-5, "weights_normalize": "mean"}),
    ("near_float_log", {"comp": "total", "nSnaps": 1, "L_screen": 1000.0,
                        "weights_normalize": "ones", "Np_max": 2}),
    ("far_log", {"comp": "spheric_complex", "nSnaps": 1}),
    ("far_double", {"comp": "total", "nSnaps": 3, "file_tracks": "tracks_with_range"}),
    ("far_double", {"comp": "total", "nSnaps": 2, "Np_max": 2,
                    "file_tracks": "tracks_without_range"}),
]


def write_track_file(h5, name, tracks, dt, it_range=None):
    """A track file in the layout the reference's converters write and
    calculate_spectrum reads (synchrad/calc.py:186-219): misc/cdt,
    misc/N_particles, optionally misc/it_range, tracks/<i>/<x..it_start>."""
    f = h5.File(name, "w")
    f["misc/cdt"] = dt
    f["misc/N_particles"] = len(tracks)
    if it_range is not None:
        f["misc/it_range"] = np.asarray(it_range)
    for i, t in enumerate(tracks):
        for c, v in zip(("x", "y", "z", "ux", "uy", "uz", "w", "it_start"), t):
            f[f"tracks/{i}/{c}"] = v
    f.close()


def prepare_track_files(h5, tracks, dt):
    write_track_file(h5, "tracks_with_range", tracks, dt, it_range=(0, 40))
    write_track_file(h5, "tracks_without_range", tracks, dt)


def h5_tracks():
    """Three short undulator tracks (8-element lists, it_start 0, 3, 5)."""
    sys.path.insert(0, str(Path(__file__).resolve().parents[2]))
    from synchrad_gb300 import workloads as wl
    tracks, dt, _ = wl.analytic_undulator_tracks(n_particles=3, n_periods=1,
                                                 steps_per_period=16, seed=5)
    out = []
    for i, t in enumerate(tracks):
        out.append([np.asarray(a)[:30 + 5 * i].copy() for a in t[:6]] + [0.5 + 0.5 * i, 2 * i])
    return out, dt


def record_h5(data, meta):
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import fake_h5py
    import ref_host_flow
    tracks, dt = h5_tracks()
    prepare_track_files(fake_h5py, tracks, dt)
    meta["h5_cases"] = []
    for i, (gname, call) in enumerate(H5_CASES):
        name = f"h5case{i}"
        in_tracks = [] if "file_tracks" in call else [list(t) for t in tracks]
        step = None if "file_tracks" in call else dt
        ref_host_flow.calculate_spectrum(dict(GRID_CASES[gname]), in_tracks,
                                         h5py_module=fake_h5py, timeStep=step,
                                         file_spectrum=name, **call)
        store = fake_h5py.FILES.pop(name)
        paths = sorted(store)
        for path in paths:
            v = store[path]
            if path.startswith("radiation/"):
                data[f"h5/{i}/{path}"] = np.array(list(v.shape) + [v.dtype.itemsize])
            else:
                data[f"h5/{i}/{path}"] = (np.array(v.decode()) if isinstance(v, bytes)
                                          else np.asarray(v))
        meta["h5_cases"].append({"grid": gname, "call": call, "paths": paths,
                                 "dt": float(dt)})


def main():
    RefCalc = load_calc_functions()
    Utilities = load_utilities()
    data = {}
    meta = {"grid_cases": GRID_CASES, "snap_cases": SNAP_CASES, "utility_cases": []}
    for name, args in GRID_CASES.items():
        obj = ref_args(RefCalc, args)
        for key in GRID_KEYS:
            if key in obj.Args:
                data[f"grid/{name}/{key}"] = np.asarray(obj.Args[key])
    for i, (gname, comp, n_snaps, sigma, L) in enumerate(RADIATION_CASES):
        obj = ref_args(RefCalc, GRID_CASES[gname])
        obj.plat_name, obj.queue = "host", None
        obj._init_data()
        for key, v in obj.Data.items():
            data[f"rad/{i}/axis/{key}"] = np.asarray(v)
        obj.Args["sigma_particle"] = obj.dtype(sigma)
        if L is not None:
            obj.Args["L_screen"] = L
        obj._init_raditaion(comp, np.uint32(n_snaps))
        data[f"rad/{i}/FormFactor"] = np.asarray(obj.Data["FormFactor"])
        if L is not None:
            data[f"rad/{i}/theta"] = np.asarray(obj.Args["theta"])
        for key, v in obj.Data["radiation"].items():
            data[f"rad/{i}/shape/{key}"] = np.array(v.shape + (np.dtype(v.dtype).itemsize,))
    meta["radiation_cases"] = RADIATION_CASES
    for i, (rng_, n) in enumerate(SNAP_CASES):
        obj = RefCalc()
        obj._set_snap_iterations(tuple(rng_), np.uint32(n))
        data[f"snaps/{i}"] = np.asarray(obj.snap_iterations)

    class RefUtil(Utilities):
        pass

    rng = np.random.default_rng(2024)
    util_cases = [("far_double", "total", ["total"]),
                  ("far_double", "cartesian", ["x", "y", "z"]),
                  ("far_double", "cartesian_complex", ["xre", "xim", "yre", "yim", "zre", "zim"]),
                  ("near_double", "total", ["total"]),
                  ("near_double", "cartesian_complex", ["xre", "xim", "yre", "yim", "zre", "zim"])]
    for ci, (gname, comp, keys) in enumerate(util_cases):
        obj = ref_args(RefCalc, GRID_CASES[gname])
        u = RefUtil()
        u.Args = obj.Args
        u.Args["comp"] = comp
        nO, nT, nP = u.Args["gridNodeNums"]
        rad = {k: rng.uniform(0.1, 2.0, size=(2, nO, nT, nP)) for k in keys}
        u.Data = {"radiation": rad}
        u.total_weight = 3.5
        filt = rng.uniform(0.5, 1.5, size=(nO, nT, nP))
        for k, v in rad.items():
            data[f"util/{ci}/in/{k}"] = v
        data[f"util/{ci}/filter"] = filt
        calls = {
            "full": lambda: u.get_full_spectrum(),
            "full_phot": lambda: u.get_full_spectrum(phot_num=True, iteration=0),
            "full_lambda_filter_norm": lambda: u.get_full_spectrum(
                lambda0_um=0.8, spect_filter=filt, normalize_to_weights=True),
            "energy_spectrum": lambda: u.get_energy_spectrum(),
            "energy": lambda: np.asarray(u.get_energy(lambda0_um=1.0)),
            "spot": lambda: u.get_spot(),
            "spot_k0": lambda: u.get_spot(k0=float(u.Args["omega"][5]) * 1.01),
            "spot_cartesian": lambda: u.get_spot_cartesian(bins=(12, 10))[0],
            "spot_cartesian_ext": lambda: u.get_spot_cartesian(bins=(12, 10))[1],
        }
        if comp.endswith("complex"):
            calls["full_x"] = lambda: u.get_full_spectrum(comp="x")
        elif comp == "cartesian":
            calls["full_y"] = lambda: u.get_full_spectrum(comp="y")
        for cname, fn in calls.items():
            data[f"util/{ci}/out/{cname}"] = np.asarray(fn())
        meta["utility_cases"].append({"grid": gname, "comp": comp, "keys": keys,
                                      "calls": sorted(calls)})
    record_h5(data, meta)
    data["meta_json"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **data)
    print(f"{OUT.name}: {len(data) - 1} arrays")


if __name__ == "__main__":
    sys.exit(main())
