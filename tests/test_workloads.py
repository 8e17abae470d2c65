"""The synthetic benchmark workloads against their stated configurations, on
the CPU: track counts, steps, grids, dtypes, work in point-steps, and the
seeded distributions (gamma, weights, step counts) they draw."""
import numpy as np

from synchrad_gb300 import workloads as wl


def _gamma0(track):
    u = np.array([np.asarray(track[k][0], dtype=np.float64) for k in (3, 4, 5)])
    return float(np.sqrt(1.0 + (u * u).sum()))


def test_far_headline_workload():
    w = wl.c2_far_mixed()
    assert len(w.tracks) == 1024 and all(t[0].size == 4000 for t in w.tracks)
    assert tuple(w.args["grid"][-1]) == (512, 64, 64) and w.args["dtype"] == "mixed"
    assert w.pt_steps == 8_587_787_108_352
    g = np.array([_gamma0(t) for t in w.tracks])
    assert abs(g.mean() / 400.0 - 1) < 1e-3 and 0.009 < g.std() / g.mean() < 0.011
    wts = np.array([t[6] for t in w.tracks])
    assert wts.min() >= 0.5 and wts.max() <= 1.5
    w1 = wl.fundamental(400.0, 1.0)
    assert np.allclose(w.args["grid"][0], (0.5 * w1, 3.5 * w1))   # first three harmonics


def test_ragged_workload():
    w = wl.c3_betatron_ragged(n_tracks=512)
    n = np.array([t[0].size for t in w.tracks])
    assert n.min() >= 500 and n.max() <= 20000 and np.unique(n).size > 400
    assert all(np.asarray(a).dtype == np.float32 for t in w.tracks for a in t[:6])
    assert tuple(w.args["grid"][-1]) == (256, 48, 48)
    g = np.array([_gamma0(t) for t in w.tracks])
    assert g.min() > 199 and g.max() < 801


def test_adjoint_workload():
    w = wl.c4_adjoint()
    assert len(w.tracks) == 256 and all(t[0].size == 2000 for t in w.tracks)
    assert tuple(w.args["grid"][-1]) == (128, 32, 32)
    assert w.pt_steps == 67_075_309_568


def test_near_workload():
    w = wl.c5_near_helical(n_tracks=256)
    assert all(t[0].size == 8000 for t in w.tracks)
    assert tuple(w.args["grid"][-1]) == (256, 64, 64) and w.args["mode"] == "near"
    assert w.pt_steps * 8 == 17_177_721_700_352          # the 2048-track workload
    assert w.L_screen == 20.0 * 50
    g = np.array([_gamma0(t) for t in w.tracks])
    assert abs(g.mean() / 300.0 - 1) < 5e-3 and 0.016 < g.std() / g.mean() < 0.024


def test_workloads_are_seeded():
    a = wl.c2_far_mixed(n_tracks=4, n_steps=100, seed=3)
    b = wl.c2_far_mixed(n_tracks=4, n_steps=100, seed=3)
    c = wl.c2_far_mixed(n_tracks=4, n_steps=100, seed=4)
    for ta, tb in zip(a.tracks, b.tracks):
        for k in range(6):
            assert np.array_equal(ta[k], tb[k])
    assert not np.array_equal(a.tracks[0][0], c.tracks[0][0])
