"""The track converters against the reference's, on the CPU.

``tests/golden/converters_golden.npz`` holds every dataset of the track files
the reference's ``tracksFromOPMD``, ``tracksFromOPMD_old`` and
``tracksFromVSIM`` (synchrad/converters.py) wrote from the synthetic inputs of
``tests/fake_openpmd.py`` through ``tests/fake_h5py.py``, and the pieces its
``split_track_by_nans`` returned on seeded NaN patterns
(``make_converter_golden.py``).  ``synchrad_gb300.converters`` must write the
same paths with the same dtypes and values, bit for bit.
"""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

import fake_h5py
import fake_openpmd
from synchrad_gb300 import converters as conv

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "converters_golden.npz")
META = json.loads(str(GOLD["meta_json"]))


@pytest.fixture
def h5(monkeypatch):
    monkeypatch.setitem(sys.modules, "h5py", fake_h5py)
    fake_h5py.FILES.clear()
    yield fake_h5py
    fake_h5py.FILES.clear()


def _compare(name):
    store = fake_h5py.FILES[name]
    exp_paths = sorted(k[len(name) + 1:] for k in GOLD.files if k.startswith(name + "/"))
    assert sorted(store) == exp_paths
    for path in exp_paths:
        exp = GOLD[f"{name}/{path}"]
        got = store[path]
        if isinstance(got, bytes):
            assert got.decode() == str(exp), path
            continue
        assert got.dtype == exp.dtype and got.shape == exp.shape, (path, got.dtype, exp.dtype)
        assert np.array_equal(got, exp, equal_nan=got.dtype.kind == "f"), path


@pytest.mark.parametrize("case", META["opmd"], ids=[c[0] for c in META["opmd"]])
def test_openpmd_track_files_match_reference(h5, case):
    name, fn, kw, seed = case
    ts, pt = fake_openpmd.scenario(gaps=(name != "opmd_xi"))
    if seed is not None:
        np.random.seed(seed)
    kw = dict(kw)
    if fn == "tracksFromOPMD_old":
        kw["verbose"] = False
    getattr(conv, fn)(ts, pt, 100, fname=name, **kw)
    _compare(name)


@pytest.mark.parametrize("case", META["vsim"], ids=[c[0] for c in META["vsim"]])
def test_vsim_track_files_match_reference(h5, case):
    name, kw = case
    f = fake_h5py.File(f"{name}_in", "w")
    f["tracks"] = fake_openpmd.vsim_tracks()
    f.close()
    conv.tracksFromVSIM(f"{name}_in", name, verbose=False, **kw)
    _compare(name)


@pytest.mark.parametrize("i", range(META["split"]))
def test_split_track_by_nans_matches_reference(i):
    cols = [GOLD[f"split/{i}/in/{k}"] for k in range(7)]
    pieces = conv.split_track_by_nans(*cols)
    assert len(pieces) == int(GOLD[f"split/{i}/n"])
    for j, piece in enumerate(pieces):
        for k, v in enumerate(piece):
            exp = GOLD[f"split/{i}/out/{j}/{k}"]
            assert np.array_equal(np.asarray(v), exp), (j, k)


def test_old_reader_list_output_feeds_calculate_spectrum():
    """Without a file name the earlier reader returns tracks in the
    [x, y, z, ux, uy, uz, w, it_start] form (the reference raises there)."""
    ts, pt = fake_openpmd.scenario()
    # weights are read at the reference iteration, 0: every one of the first
    # five particles is present there
    tracks, cdt = conv.tracksFromOPMD_old(ts, pt, 0, Np_select=5, verbose=False)
    assert cdt > 0 and len(tracks) > 0
    for t in tracks:
        assert len(t) == 8 and all(a.size == t[0].size >= 8 for a in t[:6])
        assert isinstance(t[7], int) and np.isfinite(t[6])


def test_track_file_reads_into_synchrad(h5):
    """A converted file is what SynchRad._read_tracks takes."""
    from synchrad_gb300.calc import SynchRad
    ts, pt = fake_openpmd.scenario()
    conv.tracksFromOPMD(ts, pt, 100, fname="converted")
    obj = SynchRad.__new__(SynchRad)
    obj.rank, obj.size, obj.dtype, obj.Args = 0, 1, np.double, {}
    tracks, it_range = obj._read_tracks("converted", None, 2, None, verbose=False)
    store = fake_h5py.FILES["converted"]
    assert len(tracks) == int(store["misc/N_particles"])
    assert tuple(it_range) == tuple(store["misc/it_range"])
    assert obj.Args["timeStep"] == store["misc/cdt"]
    assert np.array_equal(tracks[0][0], store["tracks/0/x"])
