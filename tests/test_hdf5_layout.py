"""HDF5 paths of SynchRad against the reference's, on the CPU.

h5py is missing here and on the GPU host, so ``tests/fake_h5py.py`` serves
the ``h5py`` calls.  ``tests/golden/host_golden.npz`` holds what the
reference's own ``calculate_spectrum`` (run by ``ref_host_flow.py`` on its
CPU-built kernels) wrote for five calls: three from track lists with
``file_spectrum`` (synchrad/calc.py:274-290) and two that also read their
tracks from a track file (synchrad/calc.py:186-219), with and without
``misc/it_range``.  The product runs the same calls with its arrays on the CPU
and the kernel call replaced by a no-op (the spectra are not the subject
here: they stay zero), and must write the same paths with the same ``Args``
values, ``snap_iterations`` and ``total_weight``, and result datasets of the
same shape and element size; ``_read_args`` must read its file back.
"""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fake_h5py  # noqa: E402
from synchrad_gb300 import calc as scalc  # noqa: E402
from synchrad_gb300.calc import SynchRad  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_host_golden as mhg  # noqa: E402

GOLD = np.load(GOLDEN / "host_golden.npz")
META = json.loads(str(GOLD["meta_json"]))


def _product(args):
    obj = SynchRad.__new__(SynchRad)
    obj.rank, obj.size = 0, 1
    a = json.loads(json.dumps(args))
    a["grid"] = [tuple(v) for v in a["grid"]]
    obj._init_args(a)
    obj.device = torch.device("cpu")
    obj._init_data()
    return obj


@pytest.fixture
def h5(monkeypatch):
    monkeypatch.setitem(sys.modules, "h5py", fake_h5py)
    monkeypatch.setattr(scalc, "run_spectrum", lambda *args, **kw: None)
    fake_h5py.FILES.clear()
    yield fake_h5py
    fake_h5py.FILES.clear()


def _run(i):
    case = META["h5_cases"][i]
    call = dict(case["call"])
    tracks, dt = mhg.h5_tracks()
    mhg.prepare_track_files(fake_h5py, tracks, dt)
    obj = _product(META["grid_cases"][case["grid"]])
    from_file = "file_tracks" in call
    obj.calculate_spectrum([] if from_file else [list(t) for t in tracks],
                           timeStep=None if from_file else dt,
                           file_spectrum=f"product{i}", verbose=False, **call)
    return obj, case, fake_h5py.FILES[f"product{i}"]


@pytest.mark.parametrize("i", range(len(META["h5_cases"])))
def test_spectrum_file_matches_reference(h5, i):
    obj, case, store = _run(i)
    assert sorted(store) == case["paths"]
    for path in case["paths"]:
        exp = GOLD[f"h5/{i}/{path}"]
        got = store[path]
        if path.startswith("radiation/"):
            assert list(got.shape) + [got.dtype.itemsize] == list(exp), path
        elif isinstance(got, bytes):
            assert got.decode() == str(exp), path
        else:
            assert got.dtype == exp.dtype and got.shape == exp.shape, (path, got.dtype, exp.dtype)
            assert np.array_equal(got, exp), path


@pytest.mark.parametrize("i", range(len(META["h5_cases"])))
def test_spectrum_file_reads_back(h5, i):
    obj, case, store = _run(i)
    back = SynchRad.__new__(SynchRad)
    back.rank, back.size = 0, 1
    back._read_args(f"product{i}")
    assert sorted(back.Data["radiation"]) == sorted(obj.Data["radiation"])
    for key, v in obj.Data["radiation"].items():
        assert np.array_equal(back.Data["radiation"][key], v)
    assert float(back.total_weight) == float(obj.total_weight)
    assert np.array_equal(back.snap_iterations, np.asarray(obj.snap_iterations))
    for key in obj.Args:
        if key in ("grid", "ctx"):
            continue
        got, exp = back.Args[key], obj.Args[key]
        if isinstance(exp, str):
            assert got == exp, key
        else:
            assert np.array_equal(np.asarray(got), np.asarray(exp)), key
