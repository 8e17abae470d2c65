"""Golden track files of the reference's converters (synchrad/converters.py).

The reference module needs h5py (and optionally numba); neither is installed,
so this script parses synchrad/converters.py from the reference tree, drops
its ``numpy`` and ``h5py`` imports and executes it with numpy (plus
``np.int``, removed from numpy 2, as the builtin ``int`` the module meant)
and ``tests/fake_h5py.py`` in their place; numba's absence selects the
module's own plain-Python fallback.  The converters then read the synthetic
inputs of ``tests/fake_openpmd.py`` and write their track files into the
stand-in, whose contents (every dataset) go to
``tests/golden/converters_golden.npz`` together with ``split_track_by_nans``
results on seeded NaN patterns.

Run from the repository root, where the reference tree is available:

    python tests/golden/make_converter_golden.py
"""
from __future__ import annotations

import ast
import os
import json
import sys
import types
import warnings
from pathlib import Path

import numpy as np

REF = Path(os.environ.get("SR_REFERENCE_ROOT", "/root/reference")) / "synchrad" / "converters.py"
TESTS = Path(__file__).resolve().parents[1]
OUT = Path(__file__).resolve().parent / "converters_golden.npz"
sys.path.insert(0, str(TESTS))

import fake_h5py  # noqa: E402
import fake_openpmd  # noqa: E402

# (name, function, keyword arguments, seed of np.random before the call)
OPMD_CASES = [
    ("opmd_all", "tracksFromOPMD", {}, None),
    # (the reference indexes its already filtered iteration list with a mask
    # of the full one when both Nit_min and Nit_max are given, and raises)
    ("opmd_random_dNp_nitmax", "tracksFromOPMD",
     {"Np_select": 6, "sample_selection": "random", "dNp": 2, "Nit_max": 300}, 3),
    ("opmd_nitmin", "tracksFromOPMD", {"Nit_min": 50}, None),
    ("opmd_sequential_short", "tracksFromOPMD",
     {"Np_select": 8, "sample_selection": "sequential", "shortest_track": 4}, None),
    ("opmd_old_first", "tracksFromOPMD_old", {"Np_select": 5}, None),
    ("opmd_old_step", "tracksFromOPMD_old", {"dNp": 2}, None),
    ("opmd_old_nit", "tracksFromOPMD_old", {"Np_select": 4, "Nit_min": 40, "Nit_max": 330},
     None),
]
# z_is_xi on particles present at every iteration (the reference's c t covers
# the whole time axis, so only full-length pieces are valid input for it)
XI_CASE = ("opmd_xi", "tracksFromOPMD", {"z_is_xi": True}, None)
VSIM_CASES = [
    ("vsim_default", {"cdt": 1.5e-7}),
    ("vsim_units_strides", {"cdt": 1.5e-7, "length_unit": 1e-6, "dNit": 2, "dNp": 2,
                            "Np_select": 3}),
]


def load_reference():
    src = REF.read_text()
    tree = ast.parse(src)
    body = []
    for n in tree.body:
        if isinstance(n, ast.Import) and any(a.name in ("numpy", "h5py") for a in n.names):
            continue
        body.append(n)
    mod = ast.Module(body=body, type_ignores=[])
    np_shim = types.ModuleType("numpy")
    np_shim.__dict__.update(np.__dict__)
    if not hasattr(np, "int"):
        np_shim.int = int
    ns = {"np": np_shim, "h5py": fake_h5py, "__name__": "reference_converters"}
    exec(compile(mod, str(REF), "exec"), ns)
    return ns


def store_file(data, prefix, name):
    for path, v in sorted(fake_h5py.FILES.pop(name).items()):
        data[f"{prefix}/{path}"] = np.array(v.decode()) if isinstance(v, bytes) else v


def main():
    ref = load_reference()
    data, meta = {}, {"opmd": [], "vsim": [], "split": 0}
    warnings.simplefilter("ignore")
    for name, fn, kw, seed in OPMD_CASES + [XI_CASE]:
        ts, pt = fake_openpmd.scenario(gaps=(name != "opmd_xi"))
        if seed is not None:
            np.random.seed(seed)
        ref[fn](ts, pt, 100, fname=name, **kw)
        store_file(data, name, name)
        meta["opmd"].append([name, fn, kw, seed])
    for name, kw in VSIM_CASES:
        f = fake_h5py.File(f"{name}_in", "w")
        f["tracks"] = fake_openpmd.vsim_tracks()
        f.close()
        ref["tracksFromVSIM"](f"{name}_in", name, verbose=False, **kw)
        fake_h5py.FILES.pop(f"{name}_in")
        store_file(data, name, name)
        meta["vsim"].append([name, kw])
    rng = np.random.default_rng(31)
    for i in range(6):
        n = int(rng.integers(1, 40))
        cols = [rng.standard_normal(n) for _ in range(6)]
        w = rng.uniform(0.5, 2.0, n)
        w[rng.random(n) < (0.1 + 0.15 * i)] = np.nan
        for k, v in enumerate(cols + [w]):
            data[f"split/{i}/in/{k}"] = v
        pieces = ref["split_track_by_nans"](*cols, w)
        data[f"split/{i}/n"] = np.array(len(pieces))
        for j, piece in enumerate(pieces):
            for k, v in enumerate(piece):
                data[f"split/{i}/out/{j}/{k}"] = np.asarray(v)
    meta["split"] = 6
    data["meta_json"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **data)
    print(f"{OUT.name}: {len(data) - 1} arrays")


if __name__ == "__main__":
    main()
