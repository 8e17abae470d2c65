"""Streaming the tracks to the device in chunks while earlier chunks compute.

``plan_chunks`` splits a batch into whole-track ranges that cover it in order
(a small leading chunk, then about equal step counts).  ``TrackStream`` packs
and copies chunk k+1 on a copy stream while chunk k is evaluated; the chunks
accumulate into one output.  On the GPU: a fixed chunking gives the same bits
as the same chunks packed and evaluated one after another, agrees with one
call over the whole batch to 1e-12 (only the FP64 order of the per-chunk sums
differs), and ``SynchRad.calculate_spectrum`` takes the chunked path for a
large batch and matches the one-call spectrum.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from synchrad_gb300 import workloads as wl  # noqa: E402
from synchrad_gb300.batch import plan_chunks  # noqa: E402


def test_plan_chunks_covers_the_batch_in_order():
    rng = np.random.default_rng(0)
    for lengths in ([4000] * 1024, rng.integers(500, 20000, 8192), [10] * 3, [5_000_000, 3]):
        plan = plan_chunks(lengths, 8)
        assert plan[0][0] == 0 and plan[-1][1] == len(lengths)
        assert all(a < b for a, b in plan)
        assert all(plan[i][1] == plan[i + 1][0] for i in range(len(plan) - 1))
    assert plan_chunks([4000] * 10, 8) == [(0, 10)]          # small: one piece
    plan = plan_chunks([4000] * 1024, 8)
    assert len(plan) == 9 and plan[0] == (0, 32)             # 1/32 leading chunk


def _grid_and_batch(w):
    from oracle import host as ohost
    from synchrad_gb300 import batch as bt
    a = ohost.init_args(dict(w.args, dtype="double"))
    n = tuple(int(v) for v in a["gridNodeNums"])
    grid = bt.make_grid("far", ohost.device_axes(a), n, torch.float64, "cuda")
    return grid, n


@pytest.mark.gpu
def test_fixed_chunking_is_reproducible_and_matches_one_call():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    w = wl.c2_far_mixed(n_tracks=64, n_steps=1500, grid=(64, 8, 8))
    grid, n = _grid_and_batch(w)
    shape = (1, n[2], n[1], n[0])
    plan = [(0, 3), (3, 30), (30, 64)]
    prec = _lib.SR_PREC_MIXED

    def streamed():
        out = torch.zeros(shape, dtype=torch.float64, device="cuda")
        ts = bt.TrackStream("cuda")
        for batch, _, _ in ts.chunks(w.tracks, np.float64, 1, w.time_step, plan=plan):
            bt.run_spectrum(batch, grid, "total", prec, [out], check_status=True)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    def sequential():
        out = torch.zeros(shape, dtype=torch.float64, device="cuda")
        for t0, t1 in plan:
            b = bt.pack_tracks(w.tracks[t0:t1], np.float64, 1, w.time_step, device="cuda")
            bt.run_spectrum(b, grid, "total", prec, [out], check_status=True)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    a, b = streamed(), sequential()
    assert np.array_equal(a, b)
    assert np.array_equal(streamed(), a)
    whole = torch.zeros(shape, dtype=torch.float64, device="cuda")
    bt.run_spectrum(bt.pack_tracks(w.tracks, np.float64, 1, w.time_step, device="cuda"), grid,
                    "total", prec, [whole], check_status=True)
    whole = whole.cpu().numpy()
    assert np.linalg.norm(a - whole) / np.linalg.norm(whole) <= 1e-12


@pytest.mark.gpu
def test_calculate_spectrum_streams_large_batches():
    """1024 tracks x 4000 steps (197 MB of FP64 coordinates: nine chunks)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    from synchrad_gb300.calc import SynchRad
    w = wl.c2_far_mixed(grid=(32, 4, 4))
    assert len(plan_chunks([len(t[0]) for t in w.tracks], 8)) > 1
    calc = SynchRad(dict(w.args))
    calc.calculate_spectrum([list(t) for t in w.tracks], timeStep=w.time_step, verbose=False)
    got = calc.Data["radiation"]["total"]
    grid, n = _grid_and_batch(w)
    ref = torch.zeros((1, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    bt.run_spectrum(bt.pack_tracks(w.tracks, np.float64, 1, w.time_step, device="cuda"), grid,
                    "total", _lib.SR_PREC_MIXED, [ref], check_status=True)
    ref = ref.cpu().numpy().swapaxes(-1, -3)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-12
    calc.calculate_spectrum([list(t) for t in w.tracks], timeStep=w.time_step, verbose=False)
    assert np.array_equal(calc.Data["radiation"]["total"], got)
