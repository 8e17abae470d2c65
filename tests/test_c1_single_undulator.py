"""The FP64 single-electron undulator case (1 electron, gamma 100, K 0.1, 20
periods + 1-period ramps at 64 steps per period = 1408 steps; grid 256 omega
over 0.5-1.5 of the fundamental x 32 theta in [0, 1/gamma] x 32 phi), the
reference's own CPU-runnable configuration, at full size.

CPU: the oracle equals the reference's kernel source compiled for the CPU bit
for bit on it, and its on-axis spectrum peaks at the undulator fundamental
2 gamma^2 / (1 + K^2/2).  GPU: SynchRad's 'double' result equals the oracle
to 1e-12 and its 'mixed' result to the mixed tolerance, 1e-5 (relative L2).
"""
import numpy as np
import pytest

import oracle
from oracle import host as ohost
from synchrad_gb300 import workloads as wl

W = wl.c1_single_undulator()
TOL_DOUBLE, TOL_MIXED = 1e-12, 1e-5


def _oracle(kind):
    rad, *_ = ohost.calculate_spectrum(dict(W.args), [list(t) for t in W.tracks], W.time_step,
                                       comp="total", kind=kind)
    return rad["total"]


def test_oracle_matches_reference_kernels_and_peaks_at_the_fundamental():
    port = _oracle("port")
    if oracle.ref_available():
        assert np.array_equal(port, _oracle("ref"))
    a = ohost.init_args(dict(W.args))
    omega = a["omega"]
    on_axis = port[0, :, 0, 0]                       # [snapshot, omega, theta, phi]
    w1 = wl.fundamental(100.0, 0.1)
    step = omega[1] - omega[0]
    assert abs(omega[int(np.argmax(on_axis))] - w1) <= 2 * step


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,tol", [("double", TOL_DOUBLE), ("mixed", TOL_MIXED)])
def test_synchrad_matches_oracle(dtype, tol):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300.calc import SynchRad
    exp = _oracle("port")
    calc = SynchRad(dict(W.args, dtype=dtype))
    calc.calculate_spectrum([list(t) for t in W.tracks], timeStep=W.time_step, comp="total",
                            verbose=False)
    got = calc.Data["radiation"]["total"]
    assert got.shape == exp.shape
    assert np.linalg.norm(got - exp) / np.linalg.norm(exp) <= tol
