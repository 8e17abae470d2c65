"""CPU checks of the C ABI: the library builds, loads without a GPU, and exports
every entry point declared in include/synchrad_gb300.h."""
import re
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def declared_entry_points():
    text = (ROOT / "include" / "synchrad_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|void|const char \*)\s*(sr_\w+)\s*\(",
                                 text, re.M)))


def test_header_declares_the_binding_table():
    from synchrad_gb300 import _lib
    assert declared_entry_points() == sorted(_lib.EXPORTS)


def test_library_loads_and_exports_every_symbol():
    from synchrad_gb300 import _lib
    L = _lib.lib()
    assert L.sr_version() >= 100
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.lib_path())],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (sr_\w+)", out))
    for name in declared_entry_points():
        assert name in exported, name
        getattr(L, name)


def test_last_error_is_empty_string_initially():
    from synchrad_gb300 import _lib
    assert _lib.lib().sr_last_error() in (b"",) or isinstance(_lib.lib().sr_last_error(), bytes)


def test_pack_tracks_csr_on_cpu():
    from synchrad_gb300.batch import pack_tracks
    tr = [[np.arange(n, dtype=np.float64) + 10 * i for _ in range(6)] + [1.5 + i, 3]
          for i, n in enumerate((5, 1, 7))]
    b = pack_tracks(tr, np.float64, 2, 0.1, device="cpu", pinned=False)
    assert b.offsets.tolist() == [0, 5, 6, 13]
    assert b.coords[0][5:6].tolist() == [10.0]
    assert b.it_end.tolist() == [5, 1, 7]
    assert b.it_start.tolist() == [0, 0, 0]
    assert b.snap_stride == 2
    assert b.snap_its.tolist() == [2, 5, 0, 1, 3, 7]
    g = pack_tracks(tr, np.float32, 3, 0.1, it_range=(0, 9), device="cpu", pinned=False)
    assert g.it_start.tolist() == [3, 3, 3] and g.it_end.tolist() == [9, 9, 9]
    assert g.snap_stride == 0 and g.snap_its.tolist() == [3, 6, 9]
    assert g.coords[0].dtype.__str__() == "torch.float32"


def test_pack_tracks_rejects_empty_track():
    import pytest
    from synchrad_gb300.batch import pack_tracks
    tr = [[np.zeros(0) for _ in range(6)] + [1.0, 0]]
    with pytest.raises(ValueError):
        pack_tracks(tr, np.float64, 1, 0.1, device="cpu", pinned=False)


def _header_signatures():
    """{name: (return kind, [parameter kinds])} parsed from the header, kinds
    being 'ptr' or the C scalar type."""
    import re
    text = (ROOT / "include" / "synchrad_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    sigs = {}
    for m in re.finditer(r"(int|int64_t|void|const char \*)\s*(sr_\w+)\s*\(([^;{]*?)\)\s*;",
                         text, re.S):
        ret, name, params = m.group(1), m.group(2), " ".join(m.group(3).split())
        kinds = []
        if params and params != "void":
            for p in params.split(","):
                p = p.strip()
                if "*" in p:
                    kinds.append("ptr")
                else:
                    kinds.append(" ".join(p.replace("const ", "").split()[:-1]))
        sigs[name] = ("ptr" if "*" in ret else ret, kinds)
    return sigs


def _ctypes_kind(t):
    import ctypes
    if t is None:
        return "void"
    if t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "_type_") and isinstance(
            getattr(t, "_type_", None), type):
        return "ptr"
    size_t = ctypes.c_size_t
    table = {ctypes.c_int: "int", ctypes.c_int64: "int64_t", ctypes.c_uint32: "uint32_t",
             ctypes.c_double: "double", size_t: "size_t"}
    for k, v in table.items():
        if t is k:
            return v
    return repr(t)


def test_binding_signatures_match_header():
    """Every ctypes argtypes/restype agrees with the header prototype: number
    of parameters, pointer or scalar, and the scalar's C type (size_t and the
    64-bit integers are the same width here, so size_t is checked by name)."""
    from synchrad_gb300 import _lib
    L = _lib.lib()
    sigs = _header_signatures()
    assert sorted(sigs) == sorted(_lib.EXPORTS)
    for name, (ret, params) in sigs.items():
        f = getattr(L, name)
        assert _ctypes_kind(f.restype) == ret, (name, f.restype, ret)
        got = [_ctypes_kind(a) for a in f.argtypes]
        assert len(got) == len(params), (name, got, params)
        for i, (g, p) in enumerate(zip(got, params)):
            if p == "size_t":
                assert g in ("size_t", "int64_t"), (name, i, g, p)
            else:
                assert g == p, (name, i, g, p)


def test_argument_errors_are_reported_before_any_device_work():
    """Invalid arguments come back as SR_ERR_INVALID with a message from the
    host-side checks, without a CUDA call (so also on a machine without a GPU)."""
    import ctypes
    from synchrad_gb300 import _lib
    L = _lib.lib()
    t, g = _lib.SrTracks(), _lib.SrGrid()
    t.n_tracks, t.total_steps, t.dtype = 1, 10, _lib.SR_DTYPE_F64
    g.n_omega, g.n_theta, g.n_phi, g.dtype = 4, 2, 2, _lib.SR_DTYPE_F64
    tp, gp = ctypes.byref(t), ctypes.byref(g)
    cases = [
        (lambda: L.sr_workspace_bytes(None, gp, 0, 3), "must not be NULL"),
        (lambda: L.sr_workspace_bytes(tp, gp, 9, 3), "unknown comp"),
        (lambda: L.sr_workspace_bytes(tp, gp, 0, 7), "unknown precision"),
    ]
    for fn, msg in cases:
        assert fn() == _lib.SR_ERR_INVALID
        assert msg in L.sr_last_error().decode()
    g.mode = _lib.SR_MODE_NEAR
    assert L.sr_workspace_bytes(tp, gp, 3, 3) == _lib.SR_ERR_INVALID
    assert "far-field only" in L.sr_last_error().decode()
    g.mode = 5
    assert L.sr_workspace_bytes(tp, gp, 0, 3) == _lib.SR_ERR_INVALID
    assert "unknown grid mode" in L.sr_last_error().decode()
    g.mode = _lib.SR_MODE_FAR
    assert L.sr_workspace_bytes(tp, gp, 0, _lib.SR_PREC_DOUBLE) == 0
    assert L.sr_workspace_bytes(tp, gp, 0, _lib.SR_PREC_MIXED) > 0
    # sr_spectrum: argument checks first
    outs = (ctypes.c_void_p * 6)()
    assert L.sr_spectrum(tp, gp, 0, 3, outs, None, 0, None) == _lib.SR_ERR_INVALID
    assert "output array 0 is NULL" in L.sr_last_error().decode()
    outs[0] = 256
    assert L.sr_spectrum(tp, gp, 0, _lib.SR_PREC_FLOAT, outs, None, 0, None) == \
        _lib.SR_ERR_INVALID
    assert "FP32 tracks and grid" in L.sr_last_error().decode()
    assert L.sr_spectrum(tp, gp, 0, 3, outs, None, 0, None) == _lib.SR_ERR_INVALID
    assert "grid axis pointer is NULL" in L.sr_last_error().decode()


def test_config_set_get_clear_on_host_fields():
    """sr_config_set pins a work shape for problems of these sizes,
    sr_config_get returns it and sr_config_clear restores the default; bad
    shapes and non-mixed precisions are refused (host fields only)."""
    import ctypes
    from synchrad_gb300 import _lib
    L = _lib.lib()
    t, g = _lib.SrTracks(), _lib.SrGrid()
    t.n_tracks, t.total_steps, t.dtype = 3, 300, _lib.SR_DTYPE_F64
    g.n_omega, g.n_theta, g.n_phi, g.dtype = 512, 4, 4, _lib.SR_DTYPE_F64
    tp, gp = ctypes.byref(t), ctypes.byref(g)
    L.sr_config_clear()
    dflt = _lib.SrConfig()
    assert L.sr_config_get(tp, gp, 0, 3, ctypes.byref(dflt)) == 0
    pin = _lib.SrConfig(16, 8, 256, 2, 0, 0, 0.0)
    assert L.sr_config_set(tp, gp, 0, 3, ctypes.byref(pin)) == 0
    got = _lib.SrConfig()
    assert L.sr_config_get(tp, gp, 0, 3, ctypes.byref(got)) == 0
    assert (got.points_per_lane, got.lanes_per_direction, got.steps_per_stage,
            got.track_subsets) == (16, 8, 256, 2)
    other = _lib.SrConfig()
    assert L.sr_config_get(tp, gp, 1, 3, ctypes.byref(other)) == 0   # another comp: default
    assert other.as_dict() == dflt.as_dict()
    assert L.sr_config_clear() == 0
    assert L.sr_config_get(tp, gp, 0, 3, ctypes.byref(got)) == 0
    assert got.as_dict() == dflt.as_dict()
    for bad in ((12, 8, 256, 0), (16, 4, 256, 0), (16, 8, 48, 0), (16, 8, 1024, 0),
                (16, 8, 256, 65)):
        assert L.sr_config_set(tp, gp, 0, 3, ctypes.byref(_lib.SrConfig(*bad, 0, 0, 0.0))) \
            == _lib.SR_ERR_INVALID, bad
    assert L.sr_config_set(tp, gp, 0, _lib.SR_PREC_DOUBLE, ctypes.byref(pin)) == \
        _lib.SR_ERR_UNSUPPORTED
    # the largest stages fit a CTA's shared memory at every lane count
    for lanes in (8, 16, 32):
        assert L.sr_config_set(tp, gp, 0, 3,
                               ctypes.byref(_lib.SrConfig(16, lanes, 512, 0, 0, 0, 0.0))) == 0
    L.sr_config_clear()
