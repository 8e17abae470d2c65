"""Host-side logic against the reference's own Python, run on the CPU.

``tests/golden/host_golden.npz`` holds what the reference's
``SynchRad._init_args`` (synchrad/calc.py:355-451), ``_set_snap_iterations``
(synchrad/calc.py:626-630) and ``Utilities`` methods (synchrad/utils.py:21-166)
return for a set of grids, snapshot ranges and seeded spectra
(``tests/golden/make_host_golden.py`` ran those function bodies from the
reference tree).  The product's host code (``synchrad_gb300.calc``,
``synchrad_gb300.batch``, ``synchrad_gb300.utils``) and the oracle's host
restatement (``oracle/host.py``) must reproduce them: bit for bit, except one
ulp on log-spaced axes, where ``np.exp``'s last bit depends on the platform;
the post-processing to 1e-13 (it sums in another order), its Cartesian spot
map on the reference's domain (values: ``tests/test_utilities.py``).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import host as ohost
from synchrad_gb300 import batch
from synchrad_gb300.calc import SynchRad

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "host_golden.npz")
META = json.loads(str(GOLD["meta_json"]))


def _product_args(args):
    obj = SynchRad.__new__(SynchRad)
    obj.rank, obj.size = 0, 1
    a = json.loads(json.dumps(args))
    a["grid"] = [tuple(v) for v in a["grid"]]
    obj._init_args(a)
    return obj


def _same(got, exp, log_axis):
    got, exp = np.asarray(got), np.asarray(exp)
    assert got.shape == exp.shape
    if log_axis and exp.dtype.kind == "f":
        np.testing.assert_array_max_ulp(got.astype(exp.dtype), exp, maxulp=2)
    else:
        assert got.dtype == exp.dtype or exp.dtype.kind != "f", (got.dtype, exp.dtype)
        assert np.array_equal(got, exp)


@pytest.mark.parametrize("name", sorted(META["grid_cases"]))
@pytest.mark.parametrize("impl", ["product", "oracle"])
def test_grid_matches_reference(name, impl):
    args = META["grid_cases"][name]
    a = _product_args(args).Args if impl == "product" else ohost.init_args(
        dict(args, grid=[tuple(v) for v in args["grid"]]))
    log_axis = "logGrid" in args.get("Features", [])
    keys = [k.split("/")[-1] for k in GOLD.files if k.startswith(f"grid/{name}/")]
    assert "omega" in keys
    for key in keys:
        _same(a[key], GOLD[f"grid/{name}/{key}"], log_axis)


@pytest.mark.parametrize("ci", range(len(META["radiation_cases"])))
def test_axes_and_result_arrays_match_reference(ci):
    """Device axes (``_init_data``), FormFactor, near-field theta and the
    result arrays' keys, shapes and element size (``_init_raditaion``); the
    product's arrays are placed on the CPU here (no kernel runs)."""
    import torch
    gname, comp, n_snaps, sigma, L = META["radiation_cases"][ci]
    args = META["grid_cases"][gname]
    log_axis = "logGrid" in args.get("Features", [])
    obj = _product_args(args)
    obj.device = torch.device("cpu")
    obj._init_data()
    ref_axes = [k.split("/")[-1] for k in GOLD.files if k.startswith(f"rad/{ci}/axis/")]
    order = (["omega", "sinTheta", "cosTheta", "sinPhi", "cosPhi"] if args.get("mode", "far") == "far"
             else ["omega", "radius", "sinPhi", "cosPhi"])
    assert sorted(ref_axes) == sorted(order)
    for key, got in zip(order, obj._host_axes):
        _same(got, GOLD[f"rad/{ci}/axis/{key}"], log_axis)
    a = ohost.init_args(dict(args, grid=[tuple(v) for v in args["grid"]]))
    for key, got in zip(order, ohost.device_axes(a)):
        _same(got, GOLD[f"rad/{ci}/axis/{key}"], log_axis)

    obj.Args["sigma_particle"] = obj.dtype(sigma)
    if L is not None:
        obj.Args["L_screen"] = L
    obj._init_raditaion(comp, np.uint32(n_snaps))
    _same(obj.Data["FormFactor"], GOLD[f"rad/{ci}/FormFactor"], log_axis)
    _same(ohost.form_factor(a, sigma), GOLD[f"rad/{ci}/FormFactor"], log_axis)
    if L is not None:
        _same(obj.Args["theta"], GOLD[f"rad/{ci}/theta"], log_axis)
    keys = [k.split("/")[-1] for k in GOLD.files if k.startswith(f"rad/{ci}/shape/")]
    assert list(obj._spect_dev) == keys
    for key, t in obj._spect_dev.items():
        exp = GOLD[f"rad/{ci}/shape/{key}"]
        assert tuple(t.shape) + (t.element_size(),) == tuple(int(v) for v in exp), key


@pytest.mark.parametrize("impl", ["product", "oracle"])
def test_snapshot_iterations_match_reference(impl):
    fn = batch.snap_iterations if impl == "product" else ohost.snap_iterations
    for i, (rng, n) in enumerate(META["snap_cases"]):
        got = fn(tuple(rng), n)
        exp = GOLD[f"snaps/{i}"]
        assert got.dtype == np.uint32 and np.array_equal(got, exp), (rng, n)


def _utility_check(ci, device=None):
    case = META["utility_cases"][ci]
    obj = _product_args(META["grid_cases"][case["grid"]])
    if device is not None:
        obj.device = device
    obj.Args["comp"] = case["comp"]
    obj.Data = {"radiation": {k: GOLD[f"util/{ci}/in/{k}"] for k in case["keys"]}}
    obj.total_weight = 3.5
    filt = GOLD[f"util/{ci}/filter"]
    calls = {
        "full": lambda: obj.get_full_spectrum(),
        "full_phot": lambda: obj.get_full_spectrum(phot_num=True, iteration=0),
        "full_lambda_filter_norm": lambda: obj.get_full_spectrum(
            lambda0_um=0.8, spect_filter=filt, normalize_to_weights=True),
        "energy_spectrum": lambda: obj.get_energy_spectrum(),
        "energy": lambda: np.asarray(obj.get_energy(lambda0_um=1.0)),
        "spot": lambda: obj.get_spot(),
        "spot_k0": lambda: obj.get_spot(k0=float(obj.Args["omega"][5]) * 1.01),
        "spot_cartesian": lambda: obj.get_spot_cartesian(bins=(12, 10))[0],
        "spot_cartesian_ext": lambda: obj.get_spot_cartesian(bins=(12, 10))[1],
        "full_x": lambda: obj.get_full_spectrum(comp="x"),
        "full_y": lambda: obj.get_full_spectrum(comp="y"),
    }
    assert set(case["calls"]) <= set(calls)
    for name in case["calls"]:
        got = np.asarray(calls[name]())
        exp = GOLD[f"util/{ci}/out/{name}"]
        assert got.shape == exp.shape, name
        if name == "spot_cartesian":
            # The reference resamples with a Delaunay triangulation of the polar
            # nodes, whose diagonal inside each cell is a tie (the four nodes
            # are co-circular); the product's own polar bilinear resampler
            # covers the same domain (the convex hull of the nodes), checked
            # here point for point, and its accuracy is checked on smooth
            # fields in tests/test_utilities.py.
            assert np.array_equal(got == 0, exp == 0), name
            continue
        np.testing.assert_allclose(got, exp, rtol=1e-13, atol=0, err_msg=name)


@pytest.mark.parametrize("ci", range(len(META["utility_cases"])))
def test_utilities_match_reference(ci):
    _utility_check(ci)


@pytest.mark.gpu
@pytest.mark.parametrize("ci", range(len(META["utility_cases"])))
def test_utilities_match_reference_on_cuda(ci):
    """The same post-processing with its torch operations on the GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _utility_check(ci, torch.device("cuda", 0))
