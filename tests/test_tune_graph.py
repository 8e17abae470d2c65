"""Batched uneven tracks: the work-shape autotuner and CUDA-graph replay.

* A graph captured from one sr_spectrum call and replayed twice accumulates
  exactly twice the direct call's spectrum (same kernels, same shape, a fixed
  summation order; doubling is exact).
* sr_autotune picks a shape among its candidates, sr_spectrum then uses it
  (sr_config_get), and the tuned result stays within the mixed-precision
  tolerance (1e-5 relative L2) of the plain FP64 kernel; sr_config_clear
  restores the default.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from synchrad_gb300 import workloads as wl  # noqa: E402

TOL_MIXED = 1e-5


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _setup(w, track_dtype=np.float64):
    from oracle import host as ohost
    from synchrad_gb300 import batch as bt
    mode = w.args.get("mode", "far")
    a = ohost.init_args(dict(w.args, dtype="double"))
    n = tuple(int(v) for v in a["gridNodeNums"])
    grid = bt.make_grid(mode, ohost.device_axes(a), n, torch.float64, "cuda",
                        L_screen=w.L_screen or 0.0)
    batch = bt.pack_tracks(w.tracks, track_dtype, 1, w.time_step, device="cuda")
    return batch, grid, n


def _spectrum(batch, grid, n, precision, ws=None):
    from synchrad_gb300 import batch as bt
    out = torch.zeros((1, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    bt.run_spectrum(batch, grid, "total", precision, [out], workspace=ws, check_status=True)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_graph_replay_equals_direct_call_ragged():
    """64 FP32 betatron tracks of 50..3000 steps in one persistent launch."""
    _need_gpu()
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    w = wl.c3_betatron_ragged(n_tracks=64, grid=(64, 12, 12), steps_range=(50, 3000))
    batch, grid, n = _setup(w, np.float32)
    direct = _spectrum(batch, grid, n, _lib.SR_PREC_MIXED)
    out = torch.zeros((1, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    g = bt.SpectrumGraph(batch, grid, "total", _lib.SR_PREC_MIXED, [out])
    k, nodes = g.nodes()
    assert k >= 3 and nodes >= k
    g.launch()
    g.launch()
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), 2.0 * direct)
    g.close()


@pytest.mark.parametrize("mode", ["far", "near"])
def test_autotune_choice_is_used_and_accurate(mode):
    _need_gpu()
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    if mode == "far":
        w = wl.c2_far_mixed(n_tracks=24, n_steps=600, grid=(96, 12, 10))
    else:
        w = wl.c5_near_helical(n_tracks=24, n_steps=800, grid=(64, 10, 8))
    batch, grid, n = _setup(w)
    _lib.lib().sr_config_clear()
    default = bt.current_config(batch, grid)
    res = bt.autotune(batch, grid, budget_ms=800.0)
    best = res["best"]
    assert res["default"]["points_per_lane"] == default["points_per_lane"]
    assert res["default"]["ms"] > 0 and best["ms"] > 0
    assert best["ms"] <= res["default"]["ms"] * 1.0001
    used = bt.current_config(batch, grid)
    for key in ("points_per_lane", "lanes_per_direction", "steps_per_stage", "track_subsets"):
        assert used[key] == best[key]
    assert best["lanes_per_direction"] in (8, 16, 32)
    if mode == "far":
        assert best["points_per_lane"] in (8, 16, 24, 32)
        assert best["steps_per_stage"] in (64, 128, 256)
    tuned = _spectrum(batch, grid, n, _lib.SR_PREC_MIXED)
    ref = _spectrum(batch, grid, n, _lib.SR_PREC_DOUBLE)
    assert _rel(tuned, ref) <= TOL_MIXED
    _lib.lib().sr_config_clear()
    assert bt.current_config(batch, grid) == default


@pytest.mark.parametrize("stage", [32, 64, 256, 512])
def test_far_stage_sizes_agree(stage):
    """Every steps-per-stage a pinned or tuned shape may use gives the same
    spectrum to rounding (the fold interval stays about 2048 steps)."""
    _need_gpu()
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    w = wl.c2_far_mixed(n_tracks=6, n_steps=1500, grid=(64, 6, 6))
    batch, grid, n = _setup(w)
    ref = _spectrum(batch, grid, n, _lib.SR_PREC_DOUBLE)
    _lib.lib().sr_config_clear()
    bt.set_config(batch, grid, points_per_lane=16, lanes_per_direction=16, steps_per_stage=stage)
    used = bt.current_config(batch, grid)
    assert used["steps_per_stage"] == stage and used["points_per_lane"] == 16
    got = _spectrum(batch, grid, n, _lib.SR_PREC_MIXED)
    _lib.lib().sr_config_clear()
    assert _rel(got, ref) <= TOL_MIXED


@pytest.mark.parametrize("K", [16, 32])
@pytest.mark.parametrize("L", [8, 16, 32])
@pytest.mark.parametrize("n_theta", [7, 12])
@pytest.mark.parametrize("case", ["included", "masked"])
def test_far_shapes_agree(K, L, n_theta, case):
    """The far-field kernel at every lane count (1, 2 or 4 directions per
    warp) stays within the mixed tolerance of the FP64 kernel: 12 theta nodes
    take the theta-group direction order (groups of 32/L neighbouring theta,
    phi first), 7 the plain order; 5 phi nodes leave the last CTA's groups
    partial; 70 omega points are no multiple of the lane tile.  "masked"
    starts the axis at 0 on coarse tracks, so the |dphase| < pi mask cuts
    through the tile on most steps (setup ballots, masked and skipped steps,
    runs of included steps)."""
    _need_gpu()
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    w = wl.c2_far_mixed(n_tracks=6, n_steps=800 if case == "included" else 150,
                        grid=(70, n_theta, 5))
    if case == "masked":
        g = list(w.args["grid"])
        g[0] = (0.0, g[0][1])
        w.args["grid"] = g
    batch, grid, n = _setup(w)
    ref = _spectrum(batch, grid, n, _lib.SR_PREC_DOUBLE)
    _lib.lib().sr_config_clear()
    bt.set_config(batch, grid, points_per_lane=K, lanes_per_direction=L, steps_per_stage=64)
    used = bt.current_config(batch, grid)
    assert used["points_per_lane"] == K and used["lanes_per_direction"] == L
    got = _spectrum(batch, grid, n, _lib.SR_PREC_MIXED)
    _lib.lib().sr_config_clear()
    assert _rel(got, ref) <= TOL_MIXED


@pytest.mark.parametrize("L", [8, 16, 32])
@pytest.mark.parametrize("case", ["included", "masked"])
def test_near_shapes_agree(L, case):
    """The near-field kernel at every lane count stays within the mixed
    tolerance of the FP64 kernel, on an omega axis that is no multiple of the
    lane tile; "masked" starts the axis at 0 on coarse tracks so the
    |dphase| < pi mask cuts through it."""
    K = 8
    _need_gpu()
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    w = wl.c5_near_helical(n_tracks=6, n_steps=800 if case == "included" else 150,
                           grid=(70, 6, 5))
    if case == "masked":
        g = list(w.args["grid"])
        g[0] = (0.0, g[0][1])
        w.args["grid"] = g
    batch, grid, n = _setup(w)
    ref = _spectrum(batch, grid, n, _lib.SR_PREC_DOUBLE)
    _lib.lib().sr_config_clear()
    bt.set_config(batch, grid, points_per_lane=K, lanes_per_direction=L, steps_per_stage=128)
    used = bt.current_config(batch, grid)
    assert used["points_per_lane"] == K and used["lanes_per_direction"] == L
    got = _spectrum(batch, grid, n, _lib.SR_PREC_MIXED)
    _lib.lib().sr_config_clear()
    assert _rel(got, ref) <= TOL_MIXED


def test_config_set_rejects_bad_shapes():
    _need_gpu()
    import ctypes
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    w = wl.c2_far_mixed(n_tracks=2, n_steps=100, grid=(32, 4, 4))
    batch, grid, n = _setup(w)
    for kw in ({"points_per_lane": 12}, {"lanes_per_direction": 4}, {"steps_per_stage": 48},
               {"steps_per_stage": 1024}, {"track_subsets": 65}):
        args = dict(points_per_lane=32, lanes_per_direction=32, steps_per_stage=128)
        args.update(kw)
        with pytest.raises(_lib.SynchRadError):
            bt.set_config(batch, grid, **args)


def test_synchrad_autotune_arg():
    """Args['autotune'] tunes once per batch size inside calculate_spectrum."""
    _need_gpu()
    from synchrad_gb300 import _lib
    from synchrad_gb300.calc import SynchRad
    _lib.lib().sr_config_clear()
    w = wl.c2_far_mixed(n_tracks=8, n_steps=400, grid=(64, 8, 8))
    tuned = SynchRad({"grid": w.args["grid"], "dtype": "mixed", "autotune": 300})
    tuned.calculate_spectrum([list(t) for t in w.tracks], timeStep=w.time_step, verbose=False)
    assert len(tuned._tuned) == 1
    tuned.calculate_spectrum([list(t) for t in w.tracks], timeStep=w.time_step, verbose=False)
    assert len(tuned._tuned) == 1  # the second call reuses the tuned shape
    ref = SynchRad({"grid": w.args["grid"], "dtype": "double"})
    ref.calculate_spectrum([list(t) for t in w.tracks], timeStep=w.time_step, verbose=False)
    got, exp = tuned.Data["radiation"]["total"], ref.Data["radiation"]["total"]
    assert _rel(got, exp) <= TOL_MIXED
    _lib.lib().sr_config_clear()
