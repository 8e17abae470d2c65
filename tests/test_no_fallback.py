"""The product path has no CPU fallback: without its CUDA library, or without a
CUDA device, it raises instead of computing anything on the host."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_missing_library_raises(monkeypatch, tmp_path):
    from synchrad_gb300 import _build, _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_build, "LIB", tmp_path / "libsynchrad_gb300.so")
    with pytest.raises(RuntimeError, match="missing or stale"):
        _lib.lib(build_if_missing=False)


def test_calculate_spectrum_without_a_gpu_raises():
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from synchrad_gb300 import workloads as wl
    from synchrad_gb300.calc import SynchRad
    tracks, dt, k_res = wl.analytic_undulator_tracks(n_particles=1, n_periods=2,
                                                     steps_per_period=8, seed=1)
    grid = [(0.5 * k_res, 1.5 * k_res), (0.0, 0.02), (0.0, 2 * np.pi), (8, 4, 4)]
    for dtype in ("double", "mixed"):
        with pytest.raises(RuntimeError, match="CUDA device"):
            calc = SynchRad({"grid": grid, "dtype": dtype})
            calc.calculate_spectrum([list(t) for t in tracks], timeStep=dt, verbose=False)
