"""Gradients of the near-field comps 'cartesian' and 'cartesian_complex'
(synchrad/kernel_nearfield.cl:106-326) through ``autograd.near_spectrum``
(``sr_near_forward_saved`` / ``sr_near_backward``).

For L = sum_k sum_p g_k(p) S_k(p) with seeded weights g_k the CUDA adjoint is
compared with autograd of the float64 PyTorch restatement (3e-6 relative L2
per group of positions, momenta and weights) and with fourth-order central
finite differences of the FP64 oracle on 16 coordinates (2e-6: the adjoint
kernel's FP32 omega sums).  The coherent
comp carries the phase of the screen distance, e^{i omega L}, and its weight
gradient follows sqrt(w).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import near_torch_ref as ntr  # noqa: E402
import oracle  # noqa: E402
from test_adjoint import pick_coordinates, rel_l2  # noqa: E402
from test_near_adjoint import concat, make_case  # noqa: E402

COMPS = ["cartesian", "cartesian_complex"]
TOL_AUTOGRAD = 3e-6
TOL_FD = 2e-6  # as for the far comps: FP32 omega sums in the adjoint kernel


def _case(comp):
    tracks, dt, axes, n, _, L, _ = make_case(True, seed=8)
    n_out = 6 if comp.endswith("_complex") else 3
    g = np.random.default_rng(41).uniform(0.5, 1.5, size=(n_out, n[2], n[1], n[0]))
    return tracks, dt, axes, n, g, L


def _oracle(track6, wp, dt, axes, n, L, comp):
    nst = track6[0].size
    n_out = 6 if comp.endswith("_complex") else 3
    spec = [np.zeros((n[2], n[1], n[0]), dtype=np.float64) for _ in range(n_out)]
    oracle.run_track("port", "near", comp, spec, [np.ascontiguousarray(a) for a in track6], wp,
                     0, nst, nst, axes, n, dt, np.array([nst], dtype=np.uint32), L_screen=L,
                     nthreads=4)
    return np.stack(spec)


def _cuda(tracks, dt, axes, n, g, L, comp):
    from synchrad_gb300.autograd import make_layout, near_spectrum
    lengths, _, coords, weights = concat(tracks)
    layout = make_layout(lengths, dt, axes, n, mode="near", L_screen=L)
    ts = [torch.tensor(c, dtype=torch.float64, device="cuda", requires_grad=True) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device="cuda", requires_grad=True)
    outs = near_spectrum(*ts, w, layout, comp)
    sum((torch.tensor(g[k], device="cuda") * o).sum() for k, o in enumerate(outs)).backward()
    torch.cuda.synchronize()
    return [t.grad.cpu().numpy() for t in ts], w.grad.cpu().numpy()


def _torch(tracks, dt, axes, g, L, comp):
    _, offsets, coords, weights = concat(tracks)
    ts = [torch.tensor(c, dtype=torch.float64, requires_grad=True) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, requires_grad=True)
    ax = [torch.tensor(a, dtype=torch.float64) for a in axes]
    fn = ntr.near_cartesian_torch if comp == "cartesian" else ntr.near_cartesian_complex_torch
    S = fn(*ts, w, offsets, dt, *ax, L)
    (torch.tensor(g) * S).sum().backward()
    return [t.grad.numpy() for t in ts], w.grad.numpy()


@pytest.mark.parametrize("comp", COMPS)
def test_near_comp_adjoint_matches_autograd(comp):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    tracks, dt, axes, n, g, L = _case(comp)
    g_ref, gw_ref = _torch(tracks, dt, axes, g, L, comp)
    g_gpu, gw_gpu = _cuda(tracks, dt, axes, n, g, L, comp)
    pos = rel_l2(np.concatenate(g_gpu[:3]), np.concatenate(g_ref[:3]))
    mom = rel_l2(np.concatenate(g_gpu[3:]), np.concatenate(g_ref[3:]))
    wts = rel_l2(gw_gpu, gw_ref)
    print(f"near {comp}: adjoint vs autograd: positions {pos:.2e}, momenta {mom:.2e}, "
          f"weights {wts:.2e}")
    assert pos <= TOL_AUTOGRAD and mom <= TOL_AUTOGRAD and wts <= TOL_AUTOGRAD


@pytest.mark.parametrize("comp", COMPS)
def test_near_comp_adjoint_matches_finite_differences(comp):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    tracks, dt, axes, n, g, L = _case(comp)
    g_gpu, _ = _cuda(tracks, dt, axes, n, g, L, comp)
    _, offsets, _, _ = concat(tracks)
    per_track = [_oracle(t[:6], t[6], dt, axes, n, L, comp) for t in tracks]
    total = sum(per_track)
    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 16, seed=43):
        base = tracks[t]
        v = base[c][s]
        h = 1e-5 * (max(1.0, abs(v)) if c >= 3 else 1.0)
        others = total - per_track[t]

        def L_of(delta):
            tr = [a.copy() for a in base[:6]]
            tr[c][s] = v + delta
            return float(np.sum(g * (others + _oracle(tr, base[6], dt, axes, n, L, comp))))

        exp.append((8.0 * (L_of(h) - L_of(-h)) - (L_of(2 * h) - L_of(-2 * h))) / (12.0 * h))
        got.append(g_gpu[c][offsets[t] + s])
    err = rel_l2(got, exp)
    print(f"near {comp}: adjoint vs finite differences (16 coordinates): {err:.2e}")
    assert err <= TOL_FD
