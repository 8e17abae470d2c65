"""The allocation-free entry point against the workspace entry point.

sr_spectrum_noalloc serves callers that cannot allocate device memory: it runs
the mixed-precision far field with its scratch in an array compiled into the
library.  Called twice in a row through the C ABI, it must give what
sr_spectrum gives with a caller-allocated workspace, within the mixed-precision
tolerance of the parity tests (1e-5 relative L2); the second call also checks
that what the first call left in the shared array does not leak into it.
sr_noalloc_status reads the static array's status word back: a clean call
reports SR_OK and a timed-out bounded wait SR_ERR_TIMEOUT.  Sizes beyond the
array and near-field grids are rejected before anything is launched.
This file is collected last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

import golden_cases as gc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5


def test_noalloc_matches_workspace_entry_point_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import host
    from synchrad_gb300 import _lib
    from synchrad_gb300.batch import make_grid, pack_tracks, run_spectrum
    L = _lib.lib()
    case = gc.load("far_cartesian_double")
    a = host.init_args(case.fresh_args())
    nsnap = int(case.call["nSnaps"])
    grid = make_grid("far", host.device_axes(a), a["gridNodeNums"], torch.float64, "cuda")
    batch = pack_tracks(case.fresh_tracks(), np.float64, nsnap, case.call["timeStep"],
                        device="cuda")
    shape = (nsnap,) + tuple(a["gridNodeNums"][::-1])
    ref = [torch.zeros(shape, dtype=torch.float64, device="cuda") for _ in range(3)]
    run_spectrum(batch, grid, "cartesian", _lib.SR_PREC_MIXED, ref, check_status=True)
    ts, gs = batch.c_struct(), grid.c_struct()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        outs = [torch.zeros(shape, dtype=torch.float64, device="cuda") for _ in range(3)]
        ptrs = (ctypes.c_void_p * 6)(*([o.data_ptr() for o in outs] + [None] * 3))
        _lib.check(L.sr_spectrum_noalloc(ctypes.byref(ts), ctypes.byref(gs),
                                         _lib.COMP_IDS["cartesian"], ptrs, stream))
        torch.cuda.synchronize()
        got = torch.cat([o.flatten() for o in outs])
        exp = torch.cat([r.flatten() for r in ref])
        rel = (torch.linalg.norm(got - exp) / torch.linalg.norm(exp)).item()
        assert rel <= TOL, f"call {call}: relative L2 {rel:.3e}"
        assert L.sr_noalloc_status(stream) == _lib.SR_OK, L.sr_last_error().decode()


def test_noalloc_status_reports_a_timed_out_wait_and_is_cleared():
    """A bounded wait that runs out in the static array's status word is what
    sr_noalloc_status reports; the next clean call clears it.  The self-test
    waits (20 ms) on an mbarrier that nothing completes: no copy, no fault."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import host
    from synchrad_gb300 import _lib
    from synchrad_gb300.batch import make_grid, pack_tracks
    L = _lib.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.sr_selftest_wait_timeout(20_000_000, None, stream))
    assert L.sr_noalloc_status(stream) == _lib.SR_ERR_TIMEOUT
    assert "ran out of time" in L.sr_last_error().decode()
    case = gc.load("far_total_double")
    a = host.init_args(case.fresh_args())
    grid = make_grid("far", host.device_axes(a), a["gridNodeNums"], torch.float64, "cuda")
    batch = pack_tracks(case.fresh_tracks(), np.float64, 1, case.call["timeStep"], device="cuda")
    out = torch.zeros((1,) + tuple(a["gridNodeNums"][::-1]), dtype=torch.float64, device="cuda")
    ptrs = (ctypes.c_void_p * 6)(out.data_ptr(), *([None] * 5))
    _lib.check(L.sr_spectrum_noalloc(ctypes.byref(batch.c_struct()), ctypes.byref(grid.c_struct()),
                                     _lib.COMP_IDS["total"], ptrs, stream))
    assert L.sr_noalloc_status(stream) == _lib.SR_OK, L.sr_last_error().decode()
    assert float(out.abs().max()) > 0.0


def test_noalloc_rejects_sizes_beyond_the_array_and_the_near_field():
    """Checked before anything is launched: the outputs stay untouched."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300 import _lib
    from synchrad_gb300.batch import make_grid, pack_tracks
    L = _lib.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = 1_000_000  # 80 MB of step records > the 64 MiB array
    z = np.linspace(0.0, 10.0, n)
    track = [np.zeros(n), np.zeros(n), z, np.zeros(n), np.zeros(n), np.full(n, 100.0), 1.0]
    batch = pack_tracks([track], np.float64, 1, 1e-5, device="cuda")
    om = 2 * np.pi * np.linspace(1.0, 2.0, 8)
    far = make_grid("far", [om, np.zeros(2), np.ones(2), np.zeros(2), np.ones(2)], (8, 2, 2),
                    torch.float64, "cuda")
    out = torch.zeros((1, 2, 2, 8), dtype=torch.float64, device="cuda")
    ptrs = (ctypes.c_void_p * 6)(out.data_ptr(), *([None] * 5))
    rc = L.sr_spectrum_noalloc(ctypes.byref(batch.c_struct()), ctypes.byref(far.c_struct()),
                               _lib.COMP_IDS["total"], ptrs, stream)
    assert rc == _lib.SR_ERR_INVALID
    assert "static array holds" in L.sr_last_error().decode()
    near = make_grid("near", [om, np.linspace(0.0, 1.0, 2), np.zeros(2), np.ones(2)], (8, 2, 2),
                     torch.float64, "cuda", L_screen=100.0)
    small = pack_tracks([[a[:100] if isinstance(a, np.ndarray) else a for a in track]],
                        np.float64, 1, 1e-5, device="cuda")
    rc = L.sr_spectrum_noalloc(ctypes.byref(small.c_struct()), ctypes.byref(near.c_struct()),
                               _lib.COMP_IDS["total"], ptrs, stream)
    assert rc == _lib.SR_ERR_UNSUPPORTED
    assert "far field only" in L.sr_last_error().decode()
    torch.cuda.synchronize()
    assert int(torch.count_nonzero(out)) == 0
