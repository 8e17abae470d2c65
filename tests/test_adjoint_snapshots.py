"""Gradients of time-resolved spectra: several snapshots per track.

The forward writes snapshot k of a track after step f_k (the reference's
state machine, synchrad/kernel_farfield.cl:53-57, 100-106), so a step enters
every snapshot written at or after it.  For L = sum_k sum_c sum_p g_k,c(p)
S_k,c(p) over three snapshots, the CUDA adjoint (``make_layout(n_snaps=3)``)
is compared with fourth-order central finite differences of the FP64 oracle,
which runs the reference's snapshot logic, on 32 coordinates: far 'total',
far 'cartesian_complex' (FormFactor applied, outputs linear in A) and near
'total'; 2e-6 relative L2 (the adjoint's FP32 omega sums), and the forward's
snapshot spectra against the oracle's at the mixed tolerance.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import oracle  # noqa: E402
from synchrad_gb300.batch import snap_iterations  # noqa: E402
from test_adjoint import concat, make_case, pick_coordinates, rel_l2  # noqa: E402

N_SNAPS = 3
TOL_FD = 2e-6
TOL_FWD = 1e-5


def _oracle(mode, comp, track6, wp, dt, axes, n, ff=None, L=0.0):
    nst = track6[0].size
    n_out = 6 if comp.endswith("_complex") else (3 if comp != "total" else 1)
    spec = [np.zeros((N_SNAPS, n[2], n[1], n[0])) for _ in range(n_out)]
    oracle.run_track("port", mode, comp, spec, [np.ascontiguousarray(a) for a in track6], wp, 0,
                     nst, nst, axes, n, dt, snap_iterations((0, nst), N_SNAPS), form_factor=ff,
                     L_screen=L, nthreads=4)
    return np.stack(spec)


def _case(mode):
    if mode == "far":
        tracks, dt, axes, n, _ = make_case(True, seed=12)
        return tracks, dt, axes, n, 0.0
    from test_near_adjoint import make_case as nmake
    tracks, dt, axes, n, _, L, _ = nmake(True, seed=13)
    return tracks, dt, axes, n, L


@pytest.mark.parametrize("mode,comp", [("far", "total"), ("far", "cartesian_complex"),
                                       ("near", "total")])
def test_snapshot_gradients_match_finite_differences(mode, comp):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300.autograd import far_spectrum, make_layout, near_spectrum
    tracks, dt, axes, n, L = _case(mode)
    ff = np.exp(-0.5 * (axes[0] / float(axes[0].max())) ** 2) if comp == "cartesian_complex" else None
    n_out = 6 if comp.endswith("_complex") else 1
    g = np.random.default_rng(51).uniform(0.5, 1.5, size=(n_out, N_SNAPS, n[2], n[1], n[0]))
    lengths, offsets, coords, weights = concat(tracks)
    layout = make_layout(lengths, dt, axes, n, mode=mode, L_screen=L, form_factor=ff,
                         n_snaps=N_SNAPS)
    ts = [torch.tensor(c, dtype=torch.float64, device="cuda", requires_grad=True) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, device="cuda", requires_grad=True)
    fn = far_spectrum if mode == "far" else near_spectrum
    outs = fn(*ts, w, layout, comp)
    assert tuple(outs[0].shape) == (N_SNAPS, n[2], n[1], n[0])
    sum((torch.tensor(g[k], device="cuda") * o).sum() for k, o in enumerate(outs)).backward()
    torch.cuda.synchronize()
    grads = [t.grad.cpu().numpy() for t in ts]

    per_track = [_oracle(mode, comp, t[:6], t[6], dt, axes, n, ff, L) for t in tracks]
    total = sum(per_track)
    got_S = np.stack([o.detach().cpu().numpy() for o in outs])
    assert rel_l2(got_S, total) <= TOL_FWD
    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 32, seed=53):
        base = tracks[t]
        v = base[c][s]
        h = 1e-5 * (max(1.0, abs(v)) if c >= 3 else 1.0)
        others = total - per_track[t]

        def L_of(delta):
            tr = [a.copy() for a in base[:6]]
            tr[c][s] = v + delta
            return float(np.sum(g * (others + _oracle(mode, comp, tr, base[6], dt, axes, n, ff, L))))

        exp.append((8.0 * (L_of(h) - L_of(-h)) - (L_of(2 * h) - L_of(-2 * h))) / (12.0 * h))
        got.append(grads[c][offsets[t] + s])
    err = rel_l2(got, exp)
    print(f"{mode} {comp}, {N_SNAPS} snapshots: adjoint vs finite differences (32 coordinates): "
          f"{err:.2e}")
    assert err <= TOL_FD
