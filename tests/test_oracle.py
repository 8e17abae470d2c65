"""The CPU oracle against the golden vectors and the reference source itself.

The golden vectors were produced by the reference's own kernel source compiled
for the CPU (tests/golden/make_golden.py).  The C restatement in
oracle/sr_oracle.c must reproduce them bit for bit (same IEEE operation order,
-ffp-contract=off, same libm); on a machine whose libm differs in the last bit
a relative tolerance of 1e-12 (FP64) is accepted instead.
"""
import platform

import numpy as np
import pytest

import oracle
from oracle import host
import golden_cases as gc

X86 = platform.machine() in ("x86_64", "AMD64")


def _check(name, got, exp, dtype):
    for key, e in exp.items():
        g = got[key]
        assert g.shape == e.shape, (name, key)
        if X86:
            assert np.array_equal(g, e), (name, key)
        else:
            tol = 1e-12 if dtype == "double" else 1e-3
            scale = max(np.abs(e).max(), 1e-300)
            assert np.abs(g - e).max() <= tol * scale, (name, key)


@pytest.mark.parametrize("name", gc.names())
def test_port_matches_golden(name):
    case = gc.load(name)
    rad, tw, snaps, _ = host.calculate_spectrum(case.fresh_args(), case.fresh_tracks(),
                                                kind="port", nthreads=2, **case.call)
    _check(name, rad, case.expected, case.args.get("dtype", "double"))
    assert tw == pytest.approx(case.total_weight, rel=1e-15)
    assert np.array_equal(snaps, case.snap_iterations)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference source not available")
@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("mode", ["far", "near"])
def test_port_matches_reference_random(seed, mode):
    """Random tracks (not smooth physics) through every kernel, both dtypes."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 40))
    tr = []
    for _ in range(2):
        x, y = 1e-3 * rng.standard_normal((2, n))
        z = np.cumsum(np.full(n, 0.02)) + 0.01 * rng.standard_normal(n)
        ux, uy = 0.3 * rng.standard_normal((2, n))
        uz = 50 + rng.standard_normal(n)
        tr.append([x, y, z, ux, uy, uz, float(rng.uniform(0.5, 2)), int(rng.integers(0, 5))])
    comps = (["total", "cartesian", "cartesian_complex", "spheric", "spheric_complex"]
             if mode == "far" else ["total", "cartesian", "cartesian_complex"])
    grid = [(0.0, 300.0), (0.0, 0.2), (0.0, 2 * np.pi), (7, 3, 4)]
    for dtype in ("double", "float"):
        for comp in comps:
            args = {"grid": grid, "dtype": dtype, "mode": mode}
            kw = dict(timeStep=0.02, comp=comp, nSnaps=int(rng.integers(1, 4)),
                      sigma_particle=1e-3, L_screen=50.0,
                      it_range=None if seed == 0 else (0, n + seed))
            cast = [[np.asarray(a, np.float32 if dtype == "float" else np.float64)
                     for a in t[:6]] + t[6:] for t in tr]
            r1 = host.calculate_spectrum(args, [list(t) for t in cast], kind="port", **kw)[0]
            r2 = host.calculate_spectrum(args, [list(t) for t in cast], kind="ref", **kw)[0]
            for k in r1:
                assert np.array_equal(r1[k], r2[k]), (mode, dtype, comp, k)


def test_oracle_rejects_wrapping_loop_bounds():
    """itEnd == 0 or nSteps == 0 would wrap the reference's unsigned loop bounds."""
    sp = [np.zeros((1, 1, 1, 2))]
    trk = [np.zeros(3) for _ in range(6)]
    axes = [np.ones(2), np.zeros(1), np.ones(1), np.zeros(1), np.ones(1)]
    with pytest.raises(ValueError):
        oracle.run_track("port", "far", "total", sp, trk, 1.0, 0, 0, 3, axes,
                         (2, 1, 1), 0.1, np.array([3], np.uint32))
    with pytest.raises(ValueError):
        oracle.run_track("port", "far", "total", sp, trk, 1.0, 0, 3, 0, axes,
                         (2, 1, 1), 0.1, np.array([3], np.uint32))


def test_snapshot_quirks_are_in_the_golden_set():
    """Repeated snapshot iterations stop the reference's snapshot index; a first
    snapshot at iteration 1 can never fire."""
    rep = gc.load("far_total_snaps_repeat")
    per_snap = np.abs(rep.expected["total"]).reshape(len(rep.snap_iterations), -1).max(1)
    assert list(rep.snap_iterations) == [2, 3, 4, 5, 5, 6, 7, 8]
    assert np.all(per_snap[1:4] > 0) and np.all(per_snap[4:] == 0)
    stuck = gc.load("far_total_snaps_stuck")
    assert stuck.snap_iterations[0] == 1
    assert np.all(stuck.expected["total"] == 0)
