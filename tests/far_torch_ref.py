"""Float64 PyTorch restatement of the reference's far-field 'total' kernel
(synchrad/kernel_farfield.cl:59-107), differentiable by autograd.

One snapshot at the end of each track (itStart = 0, itEnd = nSteps = track
length, itSnaps = [length]).  The |dphase| < pi mask is computed from the
phases and then held fixed (no gradient flows through a step function), as
the CUDA adjoint does.  Test infrastructure only.
"""
from __future__ import annotations

import math

import torch


def directions(sinT, cosT, sinP, cosP):
    """[nPhi * nTheta, 3] unit vectors, direction index iPhi * nTheta + iTheta."""
    n0 = (sinT[None, :] * cosP[:, None]).reshape(-1)
    n1 = (sinT[None, :] * sinP[:, None]).reshape(-1)
    n2 = cosT[None, :].expand(sinP.numel(), sinT.numel()).reshape(-1)
    return n0, n1, n2


def _far_track_sums(x, y, z, ux, uy, uz, offsets, dt, omega, N, n0, n1, n2):
    """Per track: (t, re, im) with re/im [nDir, nOmega, 3] the Cartesian
    components of the masked sum (synchrad/kernel_farfield.cl:59-107)."""
    for t in range(len(offsets) - 1):
        a0, a1 = int(offsets[t]), int(offsets[t + 1])
        if a1 - a0 < 2:
            continue
        X = torch.stack([x[a0:a1], y[a0:a1], z[a0:a1]], -1)
        U = torch.stack([ux[a0:a1], uy[a0:a1], uz[a0:a1]], -1)
        B = U / torch.sqrt(1.0 + (U * U).sum(-1, keepdim=True))
        acc = (B[1:] - B[:-1]) / dt
        bb = 0.5 * (B[1:] + B[:-1])
        m = a1 - a0 - 1
        time = torch.arange(m, dtype=torch.float64, device=x.device) * dt
        Xm = X[:-1]
        dotxn = (Xm[:, 0:1] * n0 + Xm[:, 1:2] * n1) + Xm[:, 2:3] * n2
        phase = omega[None, None, :] * (time[:, None, None] - dotxn[..., None])
        with torch.no_grad():
            prev = torch.cat([torch.zeros_like(phase[:1]), phase[:-1]], 0)
            mask = (phase - prev).abs() < math.pi
        c2 = 1.0 / (1.0 - bb @ N.T)
        c1 = (acc @ N.T) * c2 * c2
        amp = c1[..., None] * (N[None] - bb[:, None, :]) - c2[..., None] * acc[:, None, :]
        cw = torch.where(mask, torch.cos(phase), torch.zeros_like(phase))
        sw = torch.where(mask, torch.sin(phase), torch.zeros_like(phase))
        re = torch.einsum("mdo,mdk->dok", cw, amp)
        im = torch.einsum("mdo,mdk->dok", sw, amp)
        yield t, re, im


def far_total_torch(x, y, z, ux, uy, uz, w, offsets, dt, omega, sinT, cosT, sinP, cosP):
    """Spectrum [nPhi, nTheta, nOmega] of the concatenated tracks (CSR ``offsets``)."""
    n0, n1, n2 = directions(sinT, cosT, sinP, cosP)
    N = torch.stack([n0, n1, n2], -1)
    S = torch.zeros(N.shape[0], omega.numel(), dtype=torch.float64, device=x.device)
    for t, re, im in _far_track_sums(x, y, z, ux, uy, uz, offsets, dt, omega, N, n0, n1, n2):
        S = S + w[t] * dt * dt * ((re * re).sum(-1) + (im * im).sum(-1))
    return S.reshape(sinP.numel(), sinT.numel(), omega.numel())


def far_comps_torch(x, y, z, ux, uy, uz, w, offsets, dt, omega, sinT, cosT, sinP, cosP,
                    comp="cartesian", form_factor=None):
    """Per-component spectra [n_out][nPhi, nTheta, nOmega]: 'cartesian' |A_x|^2,
    |A_y|^2, |A_z|^2 (synchrad/kernel_farfield.cl:166-223) or 'spheric'
    |A_r|^2, |A_theta|^2, |A_phi|^2 on r = n, theta-hat = (cos theta cos phi,
    cos theta sin phi, -sin theta), phi-hat = (-sin phi, cos phi, 0)
    (:382-388, 442-445), each times w dt^2 and summed over tracks; the
    coherent 'cartesian_complex' (times the FormFactor, :283-324) and
    'spheric_complex' (:548-593) give Re and Im of each component times
    sqrt(w) dt, summed over tracks (6 outputs: re, im per component)."""
    n0, n1, n2 = directions(sinT, cosT, sinP, cosP)
    N = torch.stack([n0, n1, n2], -1)
    coherent = comp.endswith("_complex")
    comp = comp[:-len("_complex")] if coherent else comp
    if comp == "cartesian":
        basis = torch.eye(3, dtype=torch.float64, device=x.device)[None].expand(N.shape[0], 3, 3)
    elif comp == "spheric":
        cT = cosT[None, :].expand(sinP.numel(), sinT.numel()).reshape(-1)
        sT = sinT[None, :].expand(sinP.numel(), sinT.numel()).reshape(-1)
        cP = cosP[:, None].expand(sinP.numel(), sinT.numel()).reshape(-1)
        sP = sinP[:, None].expand(sinP.numel(), sinT.numel()).reshape(-1)
        th = torch.stack([cT * cP, cT * sP, -sT], -1)
        ph = torch.stack([-sP, cP, torch.zeros_like(sP)], -1)
        basis = torch.stack([N, th, ph], 1)  # [nDir, comp, xyz]
    else:
        raise ValueError(comp)
    n_out = 6 if coherent else 3
    S = torch.zeros(n_out, N.shape[0], omega.numel(), dtype=torch.float64, device=x.device)
    ff = None
    if coherent and comp == "cartesian" and form_factor is not None:
        ff = form_factor[None, None, :]
    for t, re, im in _far_track_sums(x, y, z, ux, uy, uz, offsets, dt, omega, N, n0, n1, n2):
        pr = torch.einsum("dok,dck->cdo", re, basis)
        pi = torch.einsum("dok,dck->cdo", im, basis)
        if coherent:
            f = torch.sqrt(w[t]) * dt
            if ff is not None:
                pr, pi = pr * ff, pi * ff
            S = S + f * torch.stack([pr, pi], 1).reshape(6, N.shape[0], omega.numel())
        else:
            S = S + w[t] * dt * dt * (pr * pr + pi * pi)
    return S.reshape(n_out, sinP.numel(), sinT.numel(), omega.numel())
