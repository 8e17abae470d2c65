"""Gradients of every far-field comp: cartesian, spheric and their coherent
``*_complex`` forms (synchrad/kernel_farfield.cl:111-595).

For a component-weighted loss L = sum_k sum_p g_k(p) S_k(p) with seeded
weights g_k, the CUDA adjoint (``autograd.far_spectrum``, ``sr_far_forward_saved``
/ ``sr_far_backward``) is compared with

* autograd of the float64 PyTorch restatement (``far_torch_ref.far_comps_torch``)
  over every coordinate, momentum and weight: 3e-6 relative L2 per group;
* fourth-order central finite differences of the FP64 oracle on 32 random
  coordinates: 2e-6 (the adjoint kernel sums over omega in FP32: its
  momentum gradients sit ~1.2e-6 from autograd for every comp, 'total'
  included).

``cartesian_complex`` carries a FormFactor that varies over the omega axis (the
reference applies it to that comp only); its outputs are linear in A, so its
weight gradient follows sqrt(w).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import far_torch_ref as ftr  # noqa: E402
import oracle  # noqa: E402
from test_adjoint import concat, make_case, pick_coordinates, rel_l2  # noqa: E402

COMPS = ["cartesian", "spheric", "cartesian_complex", "spheric_complex"]
TOL_AUTOGRAD = 3e-6
TOL_FD = 2e-6  # the mixed adjoint's FP32 omega sums: momenta ~1.2e-6 against autograd
TOL_FWD = 1e-5


def _case(comp):
    tracks, dt, axes, n, _ = make_case(True, seed=7)
    n_out = 6 if comp.endswith("_complex") else 3
    rng = np.random.default_rng(31)
    g = rng.uniform(0.5, 1.5, size=(n_out, n[2], n[1], n[0]))
    sigma = 1.0 / float(axes[0].max())  # FormFactor exp(-(omega sigma)^2 / 2) in [0.6, 1]
    ff = np.exp(-0.5 * (axes[0] * sigma) ** 2)
    return tracks, dt, axes, n, g, ff


def _oracle_comp(track6, wp, dt, axes, n, comp, ff):
    nst = track6[0].size
    n_out = 6 if comp.endswith("_complex") else 3
    spec = [np.zeros((n[2], n[1], n[0]), dtype=np.float64) for _ in range(n_out)]
    oracle.run_track("port", "far", comp, spec, [np.ascontiguousarray(a) for a in track6], wp,
                     0, nst, nst, axes, n, dt, np.array([nst], dtype=np.uint32),
                     form_factor=ff, nthreads=4)
    return np.stack(spec)


def _cuda(tracks, dt, axes, n, g, ff, comp):
    from synchrad_gb300.autograd import far_spectrum, make_layout
    lengths, _, coords, weights = concat(tracks)
    layout = make_layout(lengths, dt, axes, n, form_factor=ff)
    ts = [torch.tensor(c, dtype=torch.float64, device="cuda", requires_grad=True) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device="cuda", requires_grad=True)
    outs = far_spectrum(*ts, w, layout, comp)
    L = sum((torch.tensor(g[k], device="cuda") * o).sum() for k, o in enumerate(outs))
    L.backward()
    torch.cuda.synchronize()
    S = np.stack([o.detach().cpu().numpy() for o in outs])
    return [t.grad.cpu().numpy() for t in ts], w.grad.cpu().numpy(), S


def _torch(tracks, dt, axes, g, ff, comp):
    _, offsets, coords, weights = concat(tracks)
    ts = [torch.tensor(c, dtype=torch.float64, requires_grad=True) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, requires_grad=True)
    ax = [torch.tensor(a, dtype=torch.float64) for a in axes]
    S = ftr.far_comps_torch(*ts, w, offsets, dt, *ax, comp=comp,
                            form_factor=torch.tensor(ff, dtype=torch.float64))
    (torch.tensor(g) * S).sum().backward()
    return [t.grad.numpy() for t in ts], w.grad.numpy(), S.detach().numpy()


@pytest.mark.parametrize("comp", COMPS)
def test_comp_adjoint_matches_autograd(comp):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    tracks, dt, axes, n, g, ff = _case(comp)
    g_ref, gw_ref, S_ref = _torch(tracks, dt, axes, g, ff, comp)
    g_gpu, gw_gpu, S_gpu = _cuda(tracks, dt, axes, n, g, ff, comp)
    keep = [k for k in range(S_ref.shape[0]) if np.abs(S_ref[k]).max() > 1e-12 * np.abs(S_ref).max()]
    assert rel_l2(S_gpu[keep], S_ref[keep]) <= TOL_FWD
    pos = rel_l2(np.concatenate(g_gpu[:3]), np.concatenate(g_ref[:3]))
    mom = rel_l2(np.concatenate(g_gpu[3:]), np.concatenate(g_ref[3:]))
    wts = rel_l2(gw_gpu, gw_ref)
    print(f"{comp}: adjoint vs autograd: positions {pos:.2e}, momenta {mom:.2e}, "
          f"weights {wts:.2e}")
    assert pos <= TOL_AUTOGRAD and mom <= TOL_AUTOGRAD and wts <= TOL_AUTOGRAD


@pytest.mark.parametrize("comp", COMPS)
def test_comp_adjoint_matches_finite_differences(comp):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    tracks, dt, axes, n, g, ff = _case(comp)
    g_gpu, _, _ = _cuda(tracks, dt, axes, n, g, ff, comp)
    _, offsets, _, _ = concat(tracks)
    per_track = [_oracle_comp(t[:6], t[6], dt, axes, n, comp, ff) for t in tracks]
    total = sum(per_track)
    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 32, seed=37):
        base = tracks[t]
        v = base[c][s]
        h = 1e-5 * (max(1.0, abs(v)) if c >= 3 else 1.0)
        others = total - per_track[t]

        def L_of(delta):
            tr = [a.copy() for a in base[:6]]
            tr[c][s] = v + delta
            return float(np.sum(g * (others + _oracle_comp(tr, base[6], dt, axes, n, comp, ff))))

        exp.append((8.0 * (L_of(h) - L_of(-h)) - (L_of(2 * h) - L_of(-2 * h))) / (12.0 * h))
        got.append(g_gpu[c][offsets[t] + s])
    err = rel_l2(got, exp)
    print(f"{comp}: adjoint vs finite differences (32 coordinates): {err:.2e}")
    assert err <= TOL_FD
