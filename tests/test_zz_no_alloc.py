"""The allocation-free entry point against the workspace entry point.

sr_spectrum_noalloc serves callers that cannot allocate device memory: it runs
the mixed-precision far field with its scratch in an array compiled into the
library.  Called twice in a row through the C ABI, it must give what
sr_spectrum gives with a caller-allocated workspace, within the mixed-precision
tolerance of the parity tests (1e-5 relative L2); the second call also checks
that what the first call left in the shared array does not leak into it.
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
