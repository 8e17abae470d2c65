"""The reference's own ``SynchRad.calculate_spectrum`` host flow, run on the CPU.

``synchrad/calc.py`` cannot be imported here (pyopencl, mako, h5py are
missing), so this module parses it from the reference tree and runs the body
of ``SynchRad`` — ``_init_args``, ``_init_data``, ``_init_raditaion``,
``calculate_spectrum``, ``_process_track``, ``_track_to_device``,
``_spectr_from_device``, ``_set_snap_iterations``, ``_get_wgs`` — as written,
with two stand-ins: the OpenCL arrays are numpy arrays (``to_device`` copies,
``.data`` is the array itself, ``.get()`` returns it) and the compiled OpenCL
program is the reference's own kernel source compiled for the CPU
(``oracle/_ref``, built by ``oracle/build_ref.sh``), called with the argument
list ``_process_track`` assembles.  Used by ``make_golden.py`` to produce the
golden spectra and to cross-check the oracle's host restatement.
"""
from __future__ import annotations

import ast
import os
import sys
import types
from pathlib import Path

import numpy as np

REF = Path(os.environ.get("SR_REFERENCE_ROOT", "/root/reference")) / "synchrad"
ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

_METHODS = ("_init_args", "_init_data", "_init_raditaion", "calculate_spectrum",
            "_process_track", "_track_to_device", "_spectr_from_device",
            "_set_snap_iterations", "_get_wgs")
_COMP_OUTPUTS = {"total": 1, "cartesian_comps": 3, "cartesian_comps_complex": 6,
                 "spheric_comps": 3, "spheric_comps_complex": 6}
_COMP_NAMES = {"total": "total", "cartesian_comps": "cartesian",
               "cartesian_comps_complex": "cartesian_complex", "spheric_comps": "spheric",
               "spheric_comps_complex": "spheric_complex"}
# interned literals: the reference compares strings with `is`
_LITERALS = {s: s for s in ("double", "float", "far", "near", "total", "cartesian",
                            "cartesian_complex", "spheric", "spheric_complex", "mean",
                            "max", "ones")}


class HostArray(np.ndarray):
    """numpy array with the two pyopencl.array attributes the host code uses."""

    @property
    def data(self):
        return self

    def get(self):
        return np.asarray(self)


class _HostArrays:
    @staticmethod
    def to_device(queue, a):
        return np.array(a).view(HostArray)

    @staticmethod
    def zeros(queue, shape, dtype):
        return np.zeros(shape, dtype=dtype).view(HostArray)


class _Program:
    """The compiled kernels: the reference's .cl source built for the CPU."""

    def __init__(self, mode):
        self.mode = mode

    def __getattr__(self, name):
        if name not in _COMP_OUTPUTS:
            raise AttributeError(name)
        n_out = _COMP_OUTPUTS[name]

        def launch(queue, global_size, local_size, *args):
            spectra = [np.asarray(a) for a in args[:n_out]]
            rest = list(args[n_out:])
            track6 = [np.asarray(a) for a in rest[:6]]
            wp, it_start, it_end, n_steps = rest[6:10]
            n_axes = 5 if self.mode == "far" else 4
            axes = [np.asarray(a) for a in rest[10:10 + n_axes]]
            k = 10 + n_axes
            L_screen = 0.0
            if self.mode == "near":
                L_screen = rest[k]
                k += 1
            grid_n = [int(v) for v in rest[k:k + 3]]
            dt, n_snaps, snaps = rest[k + 3:k + 6]
            ff = np.asarray(rest[k + 6]) if len(rest) > k + 6 else None
            assert int(n_snaps) == np.asarray(snaps).size or int(n_snaps) <= np.asarray(snaps).size
            oracle.run_track("ref", self.mode, _COMP_NAMES[name], spectra, track6, wp,
                             it_start, it_end, n_steps, axes, grid_n, dt, np.asarray(snaps),
                             form_factor=ff, L_screen=L_screen, nthreads=4)
        return launch


def _load_class():
    src = (REF / "calc.py").read_text()
    tree = ast.parse(src)
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "SynchRad")
    funcs = [n for n in cls.body if isinstance(n, ast.FunctionDef) and n.name in _METHODS]
    assert sorted(f.name for f in funcs) == sorted(_METHODS)
    kw = {"type_params": []} if "type_params" in ast.ClassDef._fields else {}
    mod = ast.Module(body=[ast.ClassDef(name="RefSynchRad", bases=[], keywords=[], body=funcs,
                                        decorator_list=[], **kw)], type_ignores=[])
    ast.fix_missing_locations(mod)
    shim = types.ModuleType("numpy")
    shim.__dict__.update(np.__dict__)
    ns = {"np": shim, "arrcl": _HostArrays, "mpi_installed": False, "h5py": None,
          "tqdm": lambda it: it}
    exec(compile(mod, str(REF / "calc.py"), "exec"), ns)
    return ns["RefSynchRad"]


_CLASS = None


def calculate_spectrum(args: dict, tracks, h5py_module=None, **call):
    """``SynchRad(args).calculate_spectrum(tracks, **call)`` by the reference's
    host code and kernels.  Returns ``(radiation, total_weight,
    snap_iterations, Args)``; ``tracks`` is used as given (the reference
    normalises weights in place).  ``h5py_module`` serves the reference's
    ``h5py`` calls when ``file_spectrum`` is given."""
    global _CLASS
    if _CLASS is None:
        _CLASS = _load_class()
    _CLASS.calculate_spectrum.__globals__["h5py"] = h5py_module
    if not oracle.ref_available():
        raise RuntimeError("oracle/_ref is not buildable here (reference tree missing)")
    obj = _CLASS()
    obj.rank, obj.size = 0, 1
    obj.plat_name, obj.dev_type, obj.queue, obj.WGS = "host", "GPU", None, 256
    a = {k: (_LITERALS.get(v, v) if isinstance(v, str) else v) for k, v in args.items()}
    obj._init_args(a)
    obj._init_data()
    obj._mapper = _Program(obj.Args["mode"])
    kw = {k: (_LITERALS.get(v, v) if isinstance(v, str) else v) for k, v in call.items()}
    obj.calculate_spectrum(tracks, verbose=False, **kw)
    snaps = np.asarray(obj.snap_iterations)
    return dict(obj.Data["radiation"]), float(obj.total_weight), snaps, obj.Args
