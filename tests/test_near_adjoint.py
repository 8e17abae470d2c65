"""Gradients of near-field (screen) losses: L = sum(g * S) and the on-screen
radiated energy E = sum(q * S) of Utilities.get_energy.

Chain of checks as for the far field (test_adjoint.py):
  * the float64 PyTorch restatement of the near-field kernel reproduces the FP64
    oracle's spectrum, and its autograd gradient agrees with finite differences
    of the oracle (CPU);
  * get_energy_weights reproduces get_energy as a weighted sum (CPU);
  * the CUDA near-field adjoint agrees with that autograd gradient and with
    finite differences of the oracle's energy on 64 coordinates (GPU).
Finite differences: fourth-order stencil, h = 1e-5 (positions) or 1e-5 |u|.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import near_torch_ref as ntr  # noqa: E402
import oracle  # noqa: E402
from oracle import host as ohost  # noqa: E402
from synchrad_gb300 import workloads as wl  # noqa: E402

TOL_TORCH_SPECTRUM = 1e-12
TOL_TORCH_FD = 1e-7
TOL_ADJ_AUTOGRAD = 3e-6
TOL_ADJ_FD = 1e-6
TOL_FWD = 1e-5


def make_case(uniform=True, seed=3, n_omega=24, lengths=None):
    """Three helical-undulator tracks of uneven length, a screen at L = 30
    (five track lengths), 24 omega points x 5 radii x 4 azimuths."""
    rng = np.random.default_rng(seed)
    dt = 1.0 / 32
    tracks = []
    for i, (g, nper) in enumerate(((10.0, 4), (10.5, 6), (9.5, 3))):
        tr = wl.undulator_track(g, 0.5, nper, dt, x0=rng.normal(0, 0.05), y0=rng.normal(0, 0.05),
                                xp=rng.normal(0, 0.01), yp=rng.normal(0, 0.01), helical=True,
                                stagger=False, weight=float(rng.uniform(0.5, 2.0)))
        if lengths is not None:
            tr = [np.ascontiguousarray(a[:lengths[i]]) for a in tr[:6]] + tr[6:]
        tracks.append(tr)
    L = 30.0
    f1 = 2 * 10.0 ** 2 / (1 + 0.5 ** 2)
    args = {"grid": [(0.3 * f1, 2.0 * f1), (0.0, 1.2 * L / 10.0), (0.0, 2 * np.pi),
                     (n_omega, 5, 4)], "mode": "near", "dtype": "double"}
    if not uniform:
        args["Features"] = ["logGrid"]
    a = ohost.init_args(args)
    axes = ohost.device_axes(a)
    n = tuple(int(v) for v in a["gridNodeNums"])
    gmat = rng.uniform(0.5, 1.5, size=(n[2], n[1], n[0]))
    return tracks, dt, axes, n, gmat, L, a


def concat(tracks):
    lengths = np.array([t[0].size for t in tracks], dtype=np.int64)
    offsets = np.concatenate([[0], np.cumsum(lengths)])
    coords = [np.concatenate([t[c] for t in tracks]) for c in range(6)]
    weights = np.array([t[6] for t in tracks], dtype=np.float64)
    return lengths, offsets, coords, weights


def oracle_track_spectrum(track6, wp, dt, axes, n, L):
    nst = track6[0].size
    spec = np.zeros((n[2], n[1], n[0]), dtype=np.float64)
    oracle.run_track("port", "near", "total", [spec], [np.ascontiguousarray(a) for a in track6],
                     wp, 0, nst, nst, axes, n, dt, np.array([nst], dtype=np.uint32),
                     L_screen=L, nthreads=4)
    return spec


def torch_spectrum(coords, weights, offsets, dt, axes, L, device="cpu", grad=False):
    ts = [torch.tensor(c, dtype=torch.float64, device=device, requires_grad=grad) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device=device, requires_grad=grad)
    ax = [torch.tensor(v, dtype=torch.float64, device=device) for v in axes]
    return ntr.near_total_torch(*ts, w, offsets, dt, *ax, L), ts, w


def torch_gradient(tracks, dt, axes, gmat, L):
    _, offsets, coords, weights = concat(tracks)
    S, ts, w = torch_spectrum(coords, weights, offsets, dt, axes, L, grad=True)
    (torch.tensor(gmat) * S).sum().backward()
    return [t.grad.numpy() for t in ts], w.grad.numpy(), S.detach().numpy()


def fd_coordinate(tracks, dt, axes, n, L, gmat, t, c, s):
    base = tracks[t]
    v = base[c][s]
    h = 1e-5 * (max(1.0, abs(v)) if c >= 3 else 1.0)

    def loss(delta):
        tr = [a.copy() for a in base[:6]]
        tr[c][s] = v + delta
        return float(np.sum(gmat * oracle_track_spectrum(tr, base[6], dt, axes, n, L)))

    return (8.0 * (loss(h) - loss(-h)) - (loss(2 * h) - loss(-2 * h))) / (12.0 * h)


def pick_coordinates(tracks, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        t = int(rng.integers(len(tracks)))
        nst = tracks[t][0].size
        c = int(rng.integers(6))
        out.append((t, c, int(rng.integers(nst - 1))))  # the last step does not enter
    return out


def rel_l2(got, exp):
    got, exp = np.asarray(got, dtype=np.float64), np.asarray(exp, dtype=np.float64)
    return float(np.linalg.norm(got - exp) / np.linalg.norm(exp))


def energy_weights_device(a):
    """q of get_energy in the device layout [nPhi, nR, nOmega]."""
    from synchrad_gb300.utils import Utilities

    class _U(Utilities):
        pass

    u = _U()
    u.Args = dict(a, comp="total")
    return np.ascontiguousarray(u.get_energy_weights(lambda0_um=1.0).transpose(2, 1, 0))


# ---------------------------------------------------------------- CPU checks

@pytest.mark.parametrize("uniform", [True, False])
def test_torch_reference_matches_oracle(uniform):
    tracks, dt, axes, n, _, L, _ = make_case(uniform)
    _, offsets, coords, weights = concat(tracks)
    S, _, _ = torch_spectrum(coords, weights, offsets, dt, axes, L)
    exp = sum(oracle_track_spectrum(t[:6], t[6], dt, axes, n, L) for t in tracks)
    assert rel_l2(S.detach().numpy(), exp) <= TOL_TORCH_SPECTRUM


def test_torch_gradient_matches_oracle_fd():
    tracks, dt, axes, n, gmat, L, _ = make_case(True)
    grads, _, _ = torch_gradient(tracks, dt, axes, gmat, L)
    _, offsets, _, _ = concat(tracks)
    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 16, seed=11):
        got.append(grads[c][offsets[t] + s])
        exp.append(fd_coordinate(tracks, dt, axes, n, L, gmat, t, c, s))
    assert rel_l2(got, exp) <= TOL_TORCH_FD


@pytest.mark.parametrize("mode", ["far", "near"])
def test_energy_weights_reproduce_get_energy(mode):
    from synchrad_gb300.utils import Utilities
    rng = np.random.default_rng(2)
    if mode == "far":
        args = {"grid": [(10.0, 50.0), (0.0, 0.1), (0.0, 2 * np.pi), (7, 6, 5)], "mode": "far"}
    else:
        args = {"grid": [(10.0, 50.0), (0.0, 3.0), (0.0, 2 * np.pi), (7, 6, 5)], "mode": "near"}
    a = ohost.init_args(args)
    S = rng.uniform(0, 1, size=(7, 6, 5))

    class _U(Utilities):
        pass

    u = _U()
    u.Args = dict(a, comp="total")
    u.Data = {"radiation": {"total": S[None]}}
    u.total_weight = 1.0
    for lam in (None, 0.8):
        e = u.get_energy(lambda0_um=lam)
        q = u.get_energy_weights(lambda0_um=lam)
        assert np.sum(q * S) == pytest.approx(e, rel=1e-13)


# ---------------------------------------------------------------- GPU checks

def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def cuda_gradient(tracks, dt, axes, n, L, gmat):
    from synchrad_gb300.autograd import make_layout, near_total_spectrum
    lengths, _, coords, weights = concat(tracks)
    layout = make_layout(lengths, dt, axes, n, mode="near", L_screen=L)
    ts = [torch.tensor(c, dtype=torch.float64, device="cuda", requires_grad=True) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device="cuda", requires_grad=True)
    S = near_total_spectrum(*ts, w, layout)
    (torch.tensor(gmat, device="cuda") * S).sum().backward()
    torch.cuda.synchronize()
    return [t.grad.cpu().numpy() for t in ts], w.grad.cpu().numpy(), S.detach().cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("uniform", [True, False])
def test_near_adjoint_matches_autograd(uniform):
    _need_gpu()
    tracks, dt, axes, n, gmat, L, _ = make_case(uniform)
    g_ref, gw_ref, S_ref = torch_gradient(tracks, dt, axes, gmat, L)
    g_gpu, gw_gpu, S_gpu = cuda_gradient(tracks, dt, axes, n, L, gmat)
    assert rel_l2(S_gpu, S_ref) <= TOL_FWD
    pos = rel_l2(np.concatenate(g_gpu[:3]), np.concatenate(g_ref[:3]))
    mom = rel_l2(np.concatenate(g_gpu[3:]), np.concatenate(g_ref[3:]))
    wts = rel_l2(gw_gpu, gw_ref)
    print(f"near adjoint vs autograd: positions {pos:.2e}, momenta {mom:.2e}, weights {wts:.2e}")
    assert pos <= TOL_ADJ_AUTOGRAD
    assert mom <= TOL_ADJ_AUTOGRAD
    assert wts <= TOL_ADJ_AUTOGRAD


@pytest.mark.gpu
def test_screen_energy_gradient_matches_finite_differences():
    """The on-screen energy of Utilities.get_energy: its weights as dL/dS."""
    _need_gpu()
    tracks, dt, axes, n, _, L, a = make_case(True, seed=5)
    q = energy_weights_device(a)
    g_gpu, _, _ = cuda_gradient(tracks, dt, axes, n, L, q)
    _, offsets, _, _ = concat(tracks)
    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 64, seed=17):
        got.append(g_gpu[c][offsets[t] + s])
        exp.append(fd_coordinate(tracks, dt, axes, n, L, q, t, c, s))
    err = rel_l2(got, exp)
    print(f"screen energy: near adjoint vs finite differences (64 coordinates): {err:.2e}")
    assert err <= TOL_ADJ_FD


@pytest.mark.gpu
def test_near_adjoint_edge_cases():
    """Tracks of 1, 2 and 257 steps; 21 omega points (padding)."""
    _need_gpu()
    tracks, dt, axes, n, gmat, L, _ = make_case(True, seed=8, n_omega=21, lengths=(1, 2, 257))
    g_ref, gw_ref, S_ref = torch_gradient(tracks, dt, axes, gmat, L)
    g_gpu, gw_gpu, S_gpu = cuda_gradient(tracks, dt, axes, n, L, gmat)
    assert rel_l2(S_gpu, S_ref) <= TOL_FWD
    _, offsets, _, _ = concat(tracks)
    for c in range(6):
        assert np.all(g_gpu[c][offsets[0]:offsets[1]] == 0.0)
    assert gw_gpu[0] == 0.0
    pos = rel_l2(np.concatenate(g_gpu[:3]), np.concatenate(g_ref[:3]))
    mom = rel_l2(np.concatenate(g_gpu[3:]), np.concatenate(g_ref[3:]))
    print(f"near edge cases vs autograd: positions {pos:.2e}, momenta {mom:.2e}")
    assert pos <= TOL_ADJ_AUTOGRAD
    assert mom <= TOL_ADJ_AUTOGRAD
    assert rel_l2(gw_gpu[1:], gw_ref[1:]) <= TOL_ADJ_AUTOGRAD


@pytest.mark.gpu
def test_near_adjoint_deterministic():
    _need_gpu()
    tracks, dt, axes, n, gmat, L, _ = make_case(True, seed=4)
    g1, w1, _ = cuda_gradient(tracks, dt, axes, n, L, gmat)
    g2, w2, _ = cuda_gradient(tracks, dt, axes, n, L, gmat)
    for c in range(6):
        assert np.array_equal(g1[c], g2[c])
    assert np.array_equal(w1, w2)
