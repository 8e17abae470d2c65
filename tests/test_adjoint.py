"""Gradients of a far-field spectrum loss, L = sum(g * S).

Chain of checks:
  * the float64 PyTorch restatement of the far-field kernel reproduces the
    FP64 oracle's spectrum (1e-12 relative L2), and its autograd gradient
    agrees with central finite differences of the oracle (CPU tests);
  * the CUDA adjoint (``synchrad_gb300.autograd``) agrees with that autograd
    gradient over every coordinate, momentum and weight, and with finite
    differences of the FP64 oracle on 64 random coordinates (GPU tests).

Finite differences use the fourth-order stencil
(8 (L(+h) - L(-h)) - (L(+2h) - L(-2h))) / 12 h with h = 1e-5 (positions) or
1e-5 |u| (momenta); the |dphase| < pi mask does not flip for these steps on
these tracks.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import far_torch_ref as ftr  # noqa: E402
import oracle  # noqa: E402
from synchrad_gb300 import workloads as wl  # noqa: E402

# Tolerances, relative L2
TOL_TORCH_SPECTRUM = 1e-12     # torch FP64 restatement vs FP64 oracle
TOL_TORCH_FD = 1e-7            # autograd of the restatement vs oracle finite differences
TOL_ADJ_AUTOGRAD = 3e-6        # mixed-precision CUDA adjoint vs autograd (per group)
TOL_ADJ_FD = 1e-6              # mixed-precision CUDA adjoint vs finite differences
TOL_FWD = 1e-5                 # its forward spectrum vs the FP64 restatement


def make_case(uniform=True, seed=3):
    """Three planar-undulator tracks of uneven length; 40 omega points
    (uniform or geometric) around the fundamental, 6 theta x 4 phi."""
    rng = np.random.default_rng(seed)
    dt = 1.0 / 32
    tracks = []
    for g, nper in ((10.0, 4), (10.5, 6), (9.5, 3)):
        tr = wl.undulator_track(g, 0.5, nper, dt, x0=rng.normal(0, 0.05), y0=rng.normal(0, 0.05),
                                xp=rng.normal(0, 0.01), yp=rng.normal(0, 0.01),
                                weight=float(rng.uniform(0.5, 2.0)))
        tracks.append(tr)
    f1 = wl.fundamental(10.0, 0.5)
    if uniform:
        om = 2 * np.pi * f1 * np.linspace(0.3, 2.6, 40)
    else:
        om = 2 * np.pi * f1 * np.geomspace(0.3, 2.6, 40)
    theta = np.linspace(0.0, 1.5 / 10.0, 6)
    phi = np.linspace(0.0, 2 * np.pi, 4, endpoint=False)
    axes = [np.ascontiguousarray(a, dtype=np.float64)
            for a in (om, np.sin(theta), np.cos(theta), np.sin(phi), np.cos(phi))]
    n = (om.size, theta.size, phi.size)
    gmat = rng.uniform(0.5, 1.5, size=(n[2], n[1], n[0]))
    return tracks, dt, axes, n, gmat


def concat(tracks):
    lengths = np.array([t[0].size for t in tracks], dtype=np.int64)
    offsets = np.concatenate([[0], np.cumsum(lengths)])
    coords = [np.concatenate([t[c] for t in tracks]) for c in range(6)]
    weights = np.array([t[6] for t in tracks], dtype=np.float64)
    return lengths, offsets, coords, weights


def oracle_track_spectrum(track6, wp, dt, axes, n):
    nst = track6[0].size
    spec = np.zeros((n[2], n[1], n[0]), dtype=np.float64)
    oracle.run_track("port", "far", "total", [spec], [np.ascontiguousarray(a) for a in track6],
                     wp, 0, nst, nst, axes, n, dt, np.array([nst], dtype=np.uint32), nthreads=4)
    return spec


def torch_spectrum(coords, weights, offsets, dt, axes, device="cpu", grad=False):
    ts = [torch.tensor(c, dtype=torch.float64, device=device, requires_grad=grad) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device=device, requires_grad=grad)
    ax = [torch.tensor(a, dtype=torch.float64, device=device) for a in axes]
    S = ftr.far_total_torch(*ts, w, offsets, dt, *ax)
    return S, ts, w


def torch_gradient(tracks, dt, axes, gmat, device="cpu"):
    lengths, offsets, coords, weights = concat(tracks)
    S, ts, w = torch_spectrum(coords, weights, offsets, dt, axes, device, grad=True)
    L = (torch.tensor(gmat, device=device) * S).sum()
    L.backward()
    return [t.grad.cpu().numpy() for t in ts], w.grad.cpu().numpy(), S.detach().cpu().numpy()


def fd_coordinate(tracks, dt, axes, n, gmat, t, c, s):
    """Fourth-order central difference of L in coordinate c of step s of track t."""
    base = tracks[t]
    v = base[c][s]
    h = 1e-5 * (max(1.0, abs(v)) if c >= 3 else 1.0)

    def loss(delta):
        tr = [a.copy() for a in base[:6]]
        tr[c][s] = v + delta
        return float(np.sum(gmat * oracle_track_spectrum(tr, base[6], dt, axes, n)))

    return (8.0 * (loss(h) - loss(-h)) - (loss(2 * h) - loss(-2 * h))) / (12.0 * h)


def pick_coordinates(tracks, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        t = int(rng.integers(len(tracks)))
        nst = tracks[t][0].size
        c = int(rng.integers(6))
        # the last step's position does not enter the sum (its gradient is 0)
        s = int(rng.integers(nst - 1 if c < 3 else nst))
        out.append((t, c, s))
    return out


def rel_l2(got, exp):
    got, exp = np.asarray(got, dtype=np.float64), np.asarray(exp, dtype=np.float64)
    return float(np.linalg.norm(got - exp) / np.linalg.norm(exp))


# ---------------------------------------------------------------- CPU checks

@pytest.mark.parametrize("uniform", [True, False])
def test_torch_reference_matches_oracle(uniform):
    tracks, dt, axes, n, _ = make_case(uniform)
    _, offsets, coords, weights = concat(tracks)
    S, _, _ = torch_spectrum(coords, weights, offsets, dt, axes)
    exp = sum(oracle_track_spectrum(t[:6], t[6], dt, axes, n) for t in tracks)
    assert rel_l2(S.numpy(), exp) <= TOL_TORCH_SPECTRUM


def test_torch_gradient_matches_oracle_fd():
    tracks, dt, axes, n, gmat = make_case(True)
    grads, gw, _ = torch_gradient(tracks, dt, axes, gmat)
    _, offsets, _, _ = concat(tracks)
    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 16, seed=11):
        got.append(grads[c][offsets[t] + s])
        exp.append(fd_coordinate(tracks, dt, axes, n, gmat, t, c, s))
    assert rel_l2(got, exp) <= TOL_TORCH_FD


# ---------------------------------------------------------------- GPU checks

def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def cuda_gradient(tracks, dt, axes, n, gmat):
    from synchrad_gb300.autograd import far_total_spectrum, make_layout
    lengths, _, coords, weights = concat(tracks)
    layout = make_layout(lengths, dt, axes, n)
    ts = [torch.tensor(c, dtype=torch.float64, device="cuda", requires_grad=True) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device="cuda", requires_grad=True)
    S = far_total_spectrum(*ts, w, layout)
    L = (torch.tensor(gmat, device="cuda") * S).sum()
    L.backward()
    torch.cuda.synchronize()
    return [t.grad.cpu().numpy() for t in ts], w.grad.cpu().numpy(), S.detach().cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("uniform", [True, False])
def test_adjoint_matches_autograd(uniform):
    _need_gpu()
    tracks, dt, axes, n, gmat = make_case(uniform)
    g_ref, gw_ref, S_ref = torch_gradient(tracks, dt, axes, gmat)
    g_gpu, gw_gpu, S_gpu = cuda_gradient(tracks, dt, axes, n, gmat)
    assert rel_l2(S_gpu, S_ref) <= TOL_FWD
    for c in range(6):
        assert np.all(np.isfinite(g_gpu[c]))
    pos = rel_l2(np.concatenate(g_gpu[:3]), np.concatenate(g_ref[:3]))
    mom = rel_l2(np.concatenate(g_gpu[3:]), np.concatenate(g_ref[3:]))
    wts = rel_l2(gw_gpu, gw_ref)
    print(f"adjoint vs autograd: positions {pos:.2e}, momenta {mom:.2e}, weights {wts:.2e}")
    assert pos <= TOL_ADJ_AUTOGRAD
    assert mom <= TOL_ADJ_AUTOGRAD
    assert wts <= TOL_ADJ_AUTOGRAD


@pytest.mark.gpu
def test_adjoint_matches_finite_differences():
    _need_gpu()
    tracks, dt, axes, n, gmat = make_case(True, seed=5)
    g_gpu, _, _ = cuda_gradient(tracks, dt, axes, n, gmat)
    _, offsets, _, _ = concat(tracks)
    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 64, seed=17):
        got.append(g_gpu[c][offsets[t] + s])
        exp.append(fd_coordinate(tracks, dt, axes, n, gmat, t, c, s))
    err = rel_l2(got, exp)
    print(f"adjoint vs finite differences (64 coordinates): {err:.2e}")
    assert err <= TOL_ADJ_FD


@pytest.mark.gpu
def test_forward_saved_equals_spectrum():
    """The adjoint's forward is the mixed far-field kernel itself."""
    _need_gpu()
    from synchrad_gb300 import batch as bt
    from synchrad_gb300.autograd import far_total_spectrum, make_layout
    tracks, dt, axes, n, _ = make_case(True)
    lengths, _, coords, weights = concat(tracks)
    layout = make_layout(lengths, dt, axes, n)
    ts = [torch.tensor(c, dtype=torch.float64, device="cuda") for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device="cuda")
    S1 = far_total_spectrum(*ts, w, layout)
    tb = bt.pack_tracks(tracks, np.float64, 1, dt, device="cuda")
    grid = bt.make_grid("far", axes, n, torch.float64, "cuda")
    S2 = torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    bt.run_spectrum(tb, grid, "total", bt.precision_id("mixed", False), [S2], check_status=True)
    torch.cuda.synchronize()
    np.testing.assert_allclose(S1.cpu().numpy(), S2.cpu().numpy(), rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_adjoint_rejects_unsupported():
    _need_gpu()
    import ctypes
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    tracks, dt, axes, n, _ = make_case(True)
    L = _lib.lib()
    tb = bt.pack_tracks(tracks, np.float64, 0, dt, device="cuda")  # no snapshot
    grid = bt.make_grid("far", axes, n, torch.float64, "cuda")
    S = torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    A = torch.zeros(len(tracks) * int(np.prod(n)) * 4, dtype=torch.float32, device="cuda")
    ts, gs = tb.c_struct(), grid.c_struct()
    rc = L.sr_far_total_forward_saved(ctypes.byref(ts), ctypes.byref(gs), S.data_ptr(),
                                      A.data_ptr(), None, ctypes.c_size_t(0), None)
    assert rc == _lib.SR_ERR_UNSUPPORTED
    tb1 = bt.pack_tracks(tracks, np.float64, 1, dt, device="cuda")
    ts1 = tb1.c_struct()
    rc = L.sr_far_total_forward_saved(ctypes.byref(ts1), ctypes.byref(gs), S.data_ptr(),
                                      None, None, ctypes.c_size_t(0), None)
    assert rc == _lib.SR_ERR_INVALID


def make_edge_case(seed=9):
    """Tracks of 1, 2, 257 and 300 steps (an empty track, a single step, a
    one-step second work item); 37 omega points (not a multiple of the
    8-point blocks); a coarse time step so that |dphase| < pi excludes the
    upper part of the omega axis on part of each track."""
    rng = np.random.default_rng(seed)
    dt = 1.0 / 8
    tracks = []
    for L, g in ((1, 10.0), (2, 10.2), (257, 9.8), (300, 10.1)):
        tr = wl.undulator_track(g, 0.5, 40, dt, x0=rng.normal(0, 0.05),
                                weight=float(rng.uniform(0.5, 2.0)))
        tracks.append([np.ascontiguousarray(a[:L]) for a in tr[:6]] + tr[6:])
    f1 = wl.fundamental(10.0, 0.5)
    om = 2 * np.pi * f1 * np.linspace(0.5, 5.0, 37)
    theta = np.linspace(0.0, 1.0 / 10.0, 3)
    phi = np.linspace(0.0, np.pi, 2, endpoint=False)
    axes = [np.ascontiguousarray(a, dtype=np.float64)
            for a in (om, np.sin(theta), np.cos(theta), np.sin(phi), np.cos(phi))]
    n = (om.size, theta.size, phi.size)
    gmat = rng.uniform(0.5, 1.5, size=(n[2], n[1], n[0]))
    return tracks, dt, axes, n, gmat


def test_edge_case_has_a_partial_mask():
    """The coarse case really exercises the per-point mask."""
    tracks, dt, axes, n, _ = make_edge_case()
    tr = tracks[3]
    nvec = np.array([axes[1][2] * axes[4][1], axes[1][2] * axes[3][1], axes[2][2]])
    time = np.arange(tr[0].size) * dt
    ph = axes[0][None, :] * (time - (tr[0] * nvec[0] + tr[1] * nvec[1] + tr[2] * nvec[2]))[:, None]
    d = np.abs(np.diff(ph, axis=0)) < np.pi
    assert 0.05 < d.mean() < 0.95


@pytest.mark.gpu
def test_adjoint_edge_cases():
    _need_gpu()
    tracks, dt, axes, n, gmat = make_edge_case()
    g_ref, gw_ref, S_ref = torch_gradient(tracks, dt, axes, gmat)
    g_gpu, gw_gpu, S_gpu = cuda_gradient(tracks, dt, axes, n, gmat)
    assert rel_l2(S_gpu, S_ref) <= TOL_FWD
    _, offsets, _, _ = concat(tracks)
    # the one-step track contributes nothing
    for c in range(6):
        assert np.all(g_gpu[c][offsets[0]:offsets[1]] == 0.0)
    assert gw_gpu[0] == 0.0
    pos = rel_l2(np.concatenate(g_gpu[:3]), np.concatenate(g_ref[:3]))
    mom = rel_l2(np.concatenate(g_gpu[3:]), np.concatenate(g_ref[3:]))
    wts = rel_l2(gw_gpu[1:], gw_ref[1:])
    print(f"edge cases vs autograd: positions {pos:.2e}, momenta {mom:.2e}, weights {wts:.2e}")
    assert pos <= TOL_ADJ_AUTOGRAD
    assert mom <= TOL_ADJ_AUTOGRAD
    assert wts <= TOL_ADJ_AUTOGRAD


@pytest.mark.gpu
def test_adjoint_deterministic():
    _need_gpu()
    tracks, dt, axes, n, gmat = make_case(True, seed=4)
    g1, w1, _ = cuda_gradient(tracks, dt, axes, n, gmat)
    g2, w2, _ = cuda_gradient(tracks, dt, axes, n, gmat)
    for c in range(6):
        assert np.array_equal(g1[c], g2[c])
    assert np.array_equal(w1, w2)


TOL_MISFIT_E2E = 1e-3  # end to end: dL/dS from the mixed spectrum (see the test)


@pytest.mark.gpu
def test_misfit_loss_matches_finite_differences():
    """The adjoint workload's loss: weighted L2 misfit L = sum(((S - T)/max T)^2)
    against the spectrum T of the same tracks with x, y and momenta perturbed
    1e-3 relative, checked against fourth-order finite differences of the FP64
    oracle on 32 coordinates.

    * adjoint kernel: dL/dS = 2 (S - T)/max(T)^2 formed from the FP64 spectrum
      and passed to the backward: TOL_ADJ_FD;
    * end to end (mixed forward, autograd of the loss, adjoint): S - T is about
      1e-3 of S, so the ~1e-6 relative error of the mixed spectrum enters
      dL/dS amplified a thousandfold: TOL_MISFIT_E2E;
    * end to end with the double-float forward (``make_layout(precision=
      'double-float')``), whose spectrum is FP64-class: TOL_ADJ_FD.
    """
    _need_gpu()
    from synchrad_gb300.autograd import far_total_spectrum, make_layout
    tracks, dt, axes, n, _ = make_case(True, seed=6)
    target = sum(oracle_track_spectrum(t[:6], t[6], dt, axes, n)
                 for t in wl.perturbed_tracks(tracks, 1e-3, seed=1))
    inv = 1.0 / target.max()
    lengths, offsets, coords, weights = concat(tracks)
    layout = make_layout(lengths, dt, axes, n)
    per_track = [oracle_track_spectrum(t[:6], t[6], dt, axes, n) for t in tracks]
    total = sum(per_track)

    layout_df = make_layout(lengths, dt, axes, n, precision="double-float")

    def gradients(grad_from_fp64, lay=layout):
        ts = [torch.tensor(c, dtype=torch.float64, device="cuda", requires_grad=True)
              for c in coords]
        w = torch.tensor(weights, dtype=torch.float64, device="cuda", requires_grad=True)
        S = far_total_spectrum(*ts, w, lay)
        if grad_from_fp64:
            S.backward(torch.tensor(2.0 * (total - target) * inv * inv, device="cuda"))
        else:
            (((S - torch.tensor(target, device="cuda")) * inv) ** 2).sum().backward()
        return [t.grad.cpu().numpy() for t in ts]

    g64, gmx, gdf = gradients(True), gradients(False), gradients(False, layout_df)
    got64, gotmx, gotdf, exp = [], [], [], []
    for (t, c, s) in pick_coordinates(tracks, 32, seed=23):
        base = tracks[t]
        v = base[c][s]
        h = 1e-5 * (max(1.0, abs(v)) if c >= 3 else 1.0)
        others = total - per_track[t]

        def L_of(delta):
            tr = [a.copy() for a in base[:6]]
            tr[c][s] = v + delta
            St = oracle_track_spectrum(tr, base[6], dt, axes, n)
            return float(np.sum(((others + St - target) * inv) ** 2))

        exp.append((8.0 * (L_of(h) - L_of(-h)) - (L_of(2 * h) - L_of(-2 * h))) / (12.0 * h))
        got64.append(g64[c][offsets[t] + s])
        gotmx.append(gmx[c][offsets[t] + s])
        gotdf.append(gdf[c][offsets[t] + s])
    e64, emx, edf = rel_l2(got64, exp), rel_l2(gotmx, exp), rel_l2(gotdf, exp)
    print(f"misfit loss vs finite differences: adjoint {e64:.2e}, end to end {emx:.2e} "
          f"(mixed forward), {edf:.2e} (double-float forward)")
    assert e64 <= TOL_ADJ_FD
    assert emx <= TOL_MISFIT_E2E
    assert edf <= TOL_ADJ_FD
