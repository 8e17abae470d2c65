"""Gradients of the adjoint workload's misfit loss at its full size.

256 undulator electrons (K = 0.5, 2000 steps each), spectrum 128 omega x 32
theta x 32 phi, loss L = sum(((S - T) / max T)^2) against the spectrum T of
the same tracks with x, y and momenta perturbed 1e-3 relative (seed 1).
Gradients with respect to positions and momenta of 64 random coordinates are
compared with fourth-order FP64 central differences of L:

* the adjoint kernel, fed dL/dS formed from the FP64 spectrum;
* end to end through ``far_total_spectrum`` with the double-float forward
  (``make_layout(precision='double-float')``) and autograd of the loss;
both to 1e-6 relative L2.  The end-to-end gradient with the mixed forward is
reported and bounded at 1e-3: S - T is about 1e-3 of S, so the mixed
spectrum's ~1e-7 error enters dL/dS amplified about a thousandfold (a mixed
spectrum error of 1.50e-7 gives 6.5e-4 here).  The double-float forward is
the path for gradients to 1e-6.

Steps: 1e-9 in z and 1e-7 in x, y (about 1e-3 rad of phase at omega ~ 7e5),
1e-5 relative in the momenta.  The finite differences re-evaluate only the
touched track, in FP64, with the
plain FP64 CUDA kernel (the reference kernel's operations in order; equal to
the CPU oracle to 1e-12 on every golden case): L(h) = sum(((S - S_t + S_t(h)
- T) / max T)^2), S and T over all tracks also in FP64.
"""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from synchrad_gb300 import workloads as wl  # noqa: E402

TOL_FD = 1e-6
TOL_MIXED_E2E = 1e-3


def _rel(got, exp):
    got, exp = np.asarray(got), np.asarray(exp)
    return float(np.linalg.norm(got - exp) / np.linalg.norm(exp))


def test_misfit_gradient_at_full_size():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    from synchrad_gb300.autograd import far_total_spectrum, make_layout
    from synchrad_gb300.calc import SynchRad
    w = wl.c4_adjoint()
    calc = SynchRad(dict(w.args, dtype="double"))
    n = tuple(int(v) for v in calc.Args["gridNodeNums"])
    axes = calc._host_axes
    grid = bt.make_grid("far", axes, n, torch.float64, "cuda")
    dt = w.time_step

    def fp64_spectrum(tracks):
        b = bt.pack_tracks(tracks, np.float64, 1, dt, device="cuda")
        out = torch.zeros((n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
        bt.run_spectrum(b, grid, "total", _lib.SR_PREC_DOUBLE, [out])
        return out

    tracks = w.tracks
    total = fp64_spectrum(tracks)
    target = fp64_spectrum(wl.perturbed_tracks(tracks, 1e-3, seed=1))
    inv = 1.0 / float(target.max())
    lengths = [t[0].size for t in tracks]
    offsets = np.concatenate([[0], np.cumsum(lengths)])
    coords = [np.concatenate([t[c] for t in tracks]) for c in range(6)]
    weights = np.array([t[6] for t in tracks], dtype=np.float64)

    def gradients(precision, grad_fp64=False):
        lay = make_layout(lengths, dt, axes, n, precision=precision)
        ts = [torch.tensor(c, dtype=torch.float64, device="cuda", requires_grad=True)
              for c in coords]
        wt = torch.tensor(weights, dtype=torch.float64, device="cuda", requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        S = far_total_spectrum(*ts, wt, lay)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        if grad_fp64:
            S.backward(2.0 * (total - target) * inv * inv)
        else:
            (((S - target) * inv) ** 2).sum().backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        err = _rel(S.detach().cpu().numpy(), total.cpu().numpy())
        print(f"{precision} forward: {1e3 * (t1 - t0):.1f} ms, backward {1e3 * (t2 - t1):.1f} ms, "
              f"spectrum vs FP64 relative L2 {err:.2e}")
        return [t.grad.cpu().numpy() for t in ts]

    g_kernel = gradients("mixed", grad_fp64=True)
    g_df = gradients("double-float")
    g_mx = gradients("mixed")

    rng = np.random.default_rng(29)
    exp, got_k, got_df, got_mx = [], [], [], []
    for _ in range(64):
        t = int(rng.integers(len(tracks)))
        c = int(rng.integers(6))
        s = int(rng.integers(lengths[t] - 1 if c < 3 else lengths[t]))
        base = tracks[t]
        v = base[c][s]
        # steps of about 1e-3 rad in the phase at the largest omega:
        # d(tau)/dz ~ 1, d(tau)/dx,y ~ sin(theta) <= 1.5/gamma
        h = 1e-9 if c == 2 else (1e-7 if c < 2 else 1e-5 * max(1.0, abs(v)))
        own = fp64_spectrum([list(base)])
        others = total - own

        def L_of(delta):
            tr = [a.copy() for a in base[:6]] + list(base[6:])
            tr[c][s] = v + delta
            St = fp64_spectrum([tr])
            return float((((others + St - target) * inv) ** 2).sum())

        exp.append((8.0 * (L_of(h) - L_of(-h)) - (L_of(2 * h) - L_of(-2 * h))) / (12.0 * h))
        k = offsets[t] + s
        got_k.append(g_kernel[c][k])
        got_df.append(g_df[c][k])
        got_mx.append(g_mx[c][k])
    e_k, e_df, e_mx = _rel(got_k, exp), _rel(got_df, exp), _rel(got_mx, exp)
    print(f"64 coordinates vs FP64 finite differences: adjoint kernel {e_k:.2e}, end to end "
          f"{e_df:.2e} (double-float forward), {e_mx:.2e} (mixed forward)")
    assert e_k <= TOL_FD
    assert e_df <= TOL_FD
    assert e_mx <= TOL_MIXED_E2E
