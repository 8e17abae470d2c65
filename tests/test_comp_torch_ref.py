"""The float64 PyTorch restatements' per-component spectra against the
oracle, on the CPU: the far-field 'cartesian' and 'spheric' spectra
(``far_torch_ref.far_comps_torch``; synchrad/kernel_farfield.cl:111-225,
346-469) with the autograd gradient of a component-weighted loss
sum_c sum_p g_c S_c against fourth-order finite differences of the oracle,
and the near-field 'cartesian' spectra (``near_torch_ref.near_cartesian_torch``;
synchrad/kernel_nearfield.cl:106-214).  Groundwork for adjoints of the
component comps: the gradients a CUDA adjoint of those comps is checked
against."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import far_torch_ref as ftr  # noqa: E402
import oracle  # noqa: E402
from test_adjoint import concat, make_case, pick_coordinates, rel_l2  # noqa: E402


def oracle_comps(track6, wp, dt, axes, n, comp):
    nst = track6[0].size
    spec = [np.zeros((n[2], n[1], n[0]), dtype=np.float64) for _ in range(3)]
    oracle.run_track("port", "far", comp, spec, [np.ascontiguousarray(a) for a in track6], wp,
                     0, nst, nst, axes, n, dt, np.array([nst], dtype=np.uint32), nthreads=4)
    return np.stack(spec)


def torch_comps(coords, weights, offsets, dt, axes, comp, grad=False):
    ts = [torch.tensor(c, dtype=torch.float64, requires_grad=grad) for c in coords]
    w = torch.tensor(weights, dtype=torch.float64, requires_grad=grad)
    ax = [torch.tensor(a, dtype=torch.float64) for a in axes]
    return ftr.far_comps_torch(*ts, w, offsets, dt, *ax, comp=comp), ts, w


@pytest.mark.parametrize("comp", ["cartesian", "spheric"])
def test_component_spectra_match_oracle(comp):
    tracks, dt, axes, n, _ = make_case(True)
    _, offsets, coords, weights = concat(tracks)
    S, _, _ = torch_comps(coords, weights, offsets, dt, axes, comp)
    exp = sum(oracle_comps(t[:6], t[6], dt, axes, n, comp) for t in tracks)
    S = S.numpy()
    scale = np.abs(exp).max()
    for c in range(3):
        if comp == "spheric" and c == 0:
            # A is transverse: the radial part is rounding noise in both
            assert np.abs(S[0]).max() < 1e-20 * scale and np.abs(exp[0]).max() < 1e-20 * scale
        else:
            assert rel_l2(S[c], exp[c]) <= 1e-12, (comp, c)


def test_component_loss_gradient_matches_oracle_fd():
    tracks, dt, axes, n, gmat = make_case(True)
    rng = np.random.default_rng(21)
    gc = rng.uniform(0.5, 1.5, size=(3,) + gmat.shape)
    lengths, offsets, coords, weights = concat(tracks)
    S, ts, w = torch_comps(coords, weights, offsets, dt, axes, "cartesian", grad=True)
    (torch.tensor(gc) * S).sum().backward()

    def loss(t, c, s, delta):
        tr = [a.copy() for a in tracks[t][:6]]
        tr[c][s] += delta
        total = 0.0
        for i, other in enumerate(tracks):
            spec = oracle_comps(tr if i == t else other[:6], other[6], dt, axes, n,
                                "cartesian")
            total += float(np.sum(gc * spec))
        return total

    got, exp = [], []
    for (t, c, s) in pick_coordinates(tracks, 10, seed=5):
        v = tracks[t][c][s]
        h = 1e-5 * (max(1.0, abs(v)) if c >= 3 else 1.0)
        fd = (8.0 * (loss(t, c, s, h) - loss(t, c, s, -h))
              - (loss(t, c, s, 2 * h) - loss(t, c, s, -2 * h))) / (12.0 * h)
        got.append(float(ts[c].grad[offsets[t] + s]))
        exp.append(fd)
    assert rel_l2(got, exp) <= 1e-7


def test_near_component_spectra_match_oracle():
    import near_torch_ref as ntr
    from test_near_adjoint import concat as nconcat, make_case as nmake_case
    tracks, dt, axes, n, _, L, _ = nmake_case(True)
    _, offsets, coords, weights = nconcat(tracks)
    ts = [torch.tensor(c, dtype=torch.float64) for c in coords]
    ax = [torch.tensor(a, dtype=torch.float64) for a in axes]
    S = ntr.near_cartesian_torch(*ts, torch.tensor(weights), offsets, dt, *ax, L).numpy()
    exp = 0
    for t in tracks:
        nst = t[0].size
        spec = [np.zeros((n[2], n[1], n[0]), dtype=np.float64) for _ in range(3)]
        oracle.run_track("port", "near", "cartesian", spec,
                         [np.ascontiguousarray(a) for a in t[:6]], t[6], 0, nst, nst, axes, n,
                         dt, np.array([nst], dtype=np.uint32), L_screen=L, nthreads=4)
        exp = exp + np.stack(spec)
    for c in range(3):
        assert rel_l2(S[c], exp[c]) <= 1e-12, c


@pytest.mark.parametrize("comp", ["cartesian_complex", "spheric_complex"])
def test_coherent_far_components_match_oracle(comp):
    """The coherent comps of the restatement (FormFactor on cartesian_complex
    only, as the reference applies it) against the oracle."""
    tracks, dt, axes, n, _ = make_case(True)
    ff = np.exp(-0.5 * (axes[0] / float(axes[0].max())) ** 2)
    _, offsets, coords, weights = concat(tracks)
    ax = [torch.tensor(a, dtype=torch.float64) for a in axes]
    S = ftr.far_comps_torch(*[torch.tensor(c) for c in coords], torch.tensor(weights), offsets,
                            dt, *ax, comp=comp, form_factor=torch.tensor(ff)).numpy()
    exp = 0
    for t in tracks:
        nst = t[0].size
        spec = [np.zeros((n[2], n[1], n[0])) for _ in range(6)]
        oracle.run_track("port", "far", comp, spec, [np.ascontiguousarray(a) for a in t[:6]],
                         t[6], 0, nst, nst, axes, n, dt, np.array([nst], dtype=np.uint32),
                         form_factor=ff, nthreads=4)
        exp = exp + np.stack(spec)
    scale = np.abs(exp).max()
    for k in range(6):
        if comp == "spheric_complex" and k < 2:  # radial: rounding noise in both
            assert np.abs(S[k]).max() < 1e-12 * scale and np.abs(exp[k]).max() < 1e-12 * scale
        else:
            assert rel_l2(S[k], exp[k]) <= 1e-12, (comp, k)


def test_coherent_near_components_match_oracle():
    import near_torch_ref as ntr
    from test_near_adjoint import concat as nconcat, make_case as nmake_case
    tracks, dt, axes, n, _, L, _ = nmake_case(True, seed=8)
    _, offsets, coords, weights = nconcat(tracks)
    S = ntr.near_cartesian_complex_torch(*[torch.tensor(c) for c in coords],
                                         torch.tensor(weights), offsets, dt,
                                         *[torch.tensor(a) for a in axes], L).numpy()
    exp = 0
    for t in tracks:
        nst = t[0].size
        spec = [np.zeros((n[2], n[1], n[0])) for _ in range(6)]
        oracle.run_track("port", "near", "cartesian_complex", spec,
                         [np.ascontiguousarray(a) for a in t[:6]], t[6], 0, nst, nst, axes, n,
                         dt, np.array([nst], dtype=np.uint32), L_screen=L, nthreads=4)
        exp = exp + np.stack(spec)
    for k in range(6):
        assert rel_l2(S[k], exp[k]) <= 1e-11, k
