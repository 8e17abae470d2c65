"""Failure detection on the GPU without a fault: the kernels' bounded waits.

Every wait of the library's kernels (mbarrier waits on staged copies) gives up
after a time limit, records SR_ERR_TIMEOUT in the workspace status word and
returns.  The self-test kernel waits on a barrier that nothing completes, with
a 20 ms limit: the host reads the timeout through sr_workspace_status, the
kernel has ended (the stream drains), and the context still runs a spectrum.
"""
import ctypes
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    from synchrad_gb300 import workloads as wl
    L = _lib.lib()
    ws = torch.zeros(256, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    t0 = time.perf_counter()
    _lib.check(L.sr_selftest_wait_timeout(20_000_000, ctypes.c_void_p(ws.data_ptr()), sp))
    rc = L.sr_workspace_status(ctypes.c_void_p(ws.data_ptr()), sp)
    elapsed = time.perf_counter() - t0
    assert rc == _lib.SR_ERR_TIMEOUT
    assert b"ran out of time" in L.sr_last_error()
    assert 0.015 < elapsed < 5.0
    # the context is intact: a normal spectrum runs and its status is clean
    w = wl.c2_far_mixed(n_tracks=2, n_steps=300, grid=(32, 4, 4))
    from oracle import host as ohost
    a = ohost.init_args(dict(w.args, dtype="double"))
    n = tuple(int(v) for v in a["gridNodeNums"])
    grid = bt.make_grid("far", ohost.device_axes(a), n, torch.float64, "cuda")
    tb = bt.pack_tracks(w.tracks, np.float64, 1, w.time_step, device="cuda")
    out = torch.zeros((1, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    bt.run_spectrum(tb, grid, "total", _lib.SR_PREC_MIXED, [out], check_status=True)
    torch.cuda.synchronize()
    assert float(out.sum()) > 0.0


def test_selftest_rejects_bad_limits():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300 import _lib
    L = _lib.lib()
    ws = torch.zeros(256, dtype=torch.uint8, device="cuda")
    for lim in (0, -5, 2_000_000_000):
        assert L.sr_selftest_wait_timeout(lim, ctypes.c_void_p(ws.data_ptr()), None) == \
            _lib.SR_ERR_INVALID
