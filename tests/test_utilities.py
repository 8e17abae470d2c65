"""The post-processing's own parts: quadrature weights and the spot resampler.

* ``get_energy_weights`` is the quadrature of ``get_energy``: sum(q * S)
  equals ``get_energy`` on the same spectrum (far and near field).
* ``get_spot_cartesian``'s polar bilinear resampler reproduces the map at its
  nodes, is 0 outside the convex hull of the nodes, and on smooth fields is at
  least as close to the field as scipy's linear scattered-data interpolation
  (``griddata``, what the reference calls, synchrad/utils.py:143-147) is.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from synchrad_gb300.calc import SynchRad  # noqa: E402
from synchrad_gb300.utils import _polar_resample  # noqa: E402


def _calc(args):
    obj = SynchRad.__new__(SynchRad)
    obj.rank, obj.size = 0, 1
    obj._init_args(dict(args))
    obj.device = torch.device("cpu")
    return obj


@pytest.mark.parametrize("mode", ["far", "near"])
def test_energy_weights_are_get_energys_quadrature(mode):
    rng = np.random.default_rng(3)
    grid = ([(1.0, 3.0), (0.0, 0.05), (0.0, 2 * np.pi), (20, 9, 7)] if mode == "far" else
            [(1.0, 3.0), (0.0, 4.0), (0.0, 2 * np.pi), (20, 9, 7)])
    obj = _calc({"grid": grid, "mode": mode, "dtype": "double"})
    obj.Args["comp"] = "total"
    S = rng.uniform(0.5, 2.0, (1, 20, 9, 7))
    obj.Data = {"radiation": {"total": S}}
    obj.total_weight = 1.0
    q = obj.get_energy_weights(lambda0_um=0.8)
    assert q.shape == (20, 9, 7)
    e = float(obj.get_energy(lambda0_um=0.8))
    assert float((q * S[0]).sum()) == pytest.approx(e, rel=1e-13)


def _smooth(x, y):
    return np.exp(-((x - 0.01) ** 2 + (y + 0.006) ** 2) / 0.015 ** 2) + 0.3 * x / 0.03


@pytest.mark.parametrize("n_th,n_ph", [(24, 32), (12, 16)])
def test_spot_resampler_against_griddata_on_smooth_fields(n_th, n_ph):
    from scipy.interpolate import griddata
    th = np.linspace(0.0, 0.03, n_th)
    ph = 2 * np.pi / n_ph * np.arange(n_ph)
    PH, TH = np.meshgrid(ph, th)
    X, Y = TH * np.cos(PH), TH * np.sin(PH)
    spot = _smooth(X, Y)
    xs = np.linspace(-0.03, 0.03, 61)
    ys = np.linspace(-0.03, 0.03, 47)
    got = _polar_resample(torch.tensor(spot), torch.tensor(th), torch.tensor(ph),
                          torch.tensor(xs), torch.tensor(ys)).numpy()
    GX, GY = np.meshgrid(xs, ys, indexing="ij")
    ref = griddata((X.ravel(), Y.ravel()), spot.ravel(), (GX.ravel(), GY.ravel()),
                   fill_value=0.0, method="linear").reshape(GX.shape)
    assert np.array_equal(got == 0, ref == 0)       # same domain (the hull)
    inside = ref != 0
    truth = _smooth(GX, GY)
    err_ours = np.abs(got - truth)[inside].max()
    err_tri = np.abs(ref - truth)[inside].max()
    assert err_ours <= 1.5 * err_tri, (err_ours, err_tri)
    assert err_ours <= 0.05 * np.abs(truth).max()


def test_spot_resampler_reproduces_nodes():
    rng = np.random.default_rng(0)
    th = np.linspace(0.0, 2.0, 9)
    ph = 2 * np.pi / 8 * np.arange(8)
    spot = rng.uniform(1.0, 2.0, (9, 8))
    spot[0, :] = spot[0, 0]  # one value at the centre, as a physical map has
    xs = np.linspace(-2.0, 2.0, 17)  # the theta nodes on both half axes
    ys = np.array([0.0])
    got = _polar_resample(torch.tensor(spot), torch.tensor(th), torch.tensor(ph),
                          torch.tensor(xs), torch.tensor(ys)).numpy()[:, 0]
    np.testing.assert_allclose(got[8:], spot[:, 0], rtol=1e-12)     # phi = 0 ray
    np.testing.assert_allclose(got[:9][::-1], spot[:, 4], rtol=1e-12)  # phi = pi ray
