"""Float64 PyTorch restatement of the reference's near-field 'total' kernel
(synchrad/kernel_nearfield.cl:58-102), differentiable by autograd.

One snapshot at the end of each track (itStart = 0, itEnd = nSteps = track
length).  The |dphase| < pi mask is computed from the phases and then held
fixed, as the CUDA adjoint does.  Test infrastructure only.
"""
from __future__ import annotations

import math

import torch


def _near_track_sums(x, y, z, ux, uy, uz, offsets, dt, omega, X0, Y0, L_screen):
    """Per track: (t, re, im) with re/im [nScreen, nOmega, 3] the Cartesian
    components of the masked sum (synchrad/kernel_nearfield.cl:58-102)."""
    for t in range(len(offsets) - 1):
        a0, a1 = int(offsets[t]), int(offsets[t + 1])
        if a1 - a0 < 2:
            continue
        m = a1 - a0 - 1  # steps 0 .. n-2 enter the sum
        xs, ys, zs = x[a0:a1 - 1], y[a0:a1 - 1], z[a0:a1 - 1]
        U = torch.stack([ux[a0:a1 - 1], uy[a0:a1 - 1], uz[a0:a1 - 1]], -1)
        B = U / torch.sqrt(1.0 + (U * U).sum(-1, keepdim=True))           # [m, 3]
        rx = X0[None, :] - xs[:, None]
        ry = Y0[None, :] - ys[:, None]
        rz = (L_screen - zs)[:, None].expand_as(rx)
        r = torch.sqrt(rx * rx + ry * ry + rz * rz)                         # [m, D]
        n = torch.stack([rx, ry, rz], -1) / r[..., None]                   # [m, D, 3]
        time = torch.arange(m, dtype=torch.float64, device=x.device) * dt
        phase = omega[None, None, :] * (time[:, None, None] + r[..., None])  # [m, D, O]
        with torch.no_grad():
            prev = torch.cat([torch.zeros_like(phase[:1]), phase[:-1]], 0)
            mask = (phase - prev).abs() < math.pi
        cw = torch.where(mask, torch.cos(phase), torch.zeros_like(phase))
        sw = torch.where(mask, torch.sin(phase), torch.zeros_like(phase))
        c2 = n / (r * r)[..., None]                                        # [m, D, 3]
        c1b = (B[:, None, :] - n) / r[..., None]                           # c1 / omega
        # Re += -omega c1b sin + c2 cos;  Im += omega c1b cos + c2 sin
        re = (torch.einsum("mdo,mdk->dok", cw, c2)
              - omega[None, :, None] * torch.einsum("mdo,mdk->dok", sw, c1b))
        im = (torch.einsum("mdo,mdk->dok", sw, c2)
              + omega[None, :, None] * torch.einsum("mdo,mdk->dok", cw, c1b))
        yield t, re, im


def _screen(radius, sinP, cosP):
    X0 = (radius[None, :] * cosP[:, None]).reshape(-1)  # screen point index iPhi * nR + iR
    Y0 = (radius[None, :] * sinP[:, None]).reshape(-1)
    return X0, Y0


def near_total_torch(x, y, z, ux, uy, uz, w, offsets, dt, omega, radius, sinP, cosP, L_screen):
    """Spectrum [nPhi, nR, nOmega] of the concatenated tracks (CSR ``offsets``)."""
    X0, Y0 = _screen(radius, sinP, cosP)
    S = torch.zeros(X0.numel(), omega.numel(), dtype=torch.float64, device=x.device)
    for t, re, im in _near_track_sums(x, y, z, ux, uy, uz, offsets, dt, omega, X0, Y0,
                                      L_screen):
        S = S + w[t] * dt * dt * ((re * re).sum(-1) + (im * im).sum(-1))
    return S.reshape(sinP.numel(), radius.numel(), omega.numel())


def near_cartesian_torch(x, y, z, ux, uy, uz, w, offsets, dt, omega, radius, sinP, cosP,
                         L_screen):
    """Per-component spectra [3][nPhi, nR, nOmega]: w dt^2 |A_x|^2, |A_y|^2,
    |A_z|^2 summed over tracks (synchrad/kernel_nearfield.cl:106-214)."""
    X0, Y0 = _screen(radius, sinP, cosP)
    S = torch.zeros(3, X0.numel(), omega.numel(), dtype=torch.float64, device=x.device)
    for t, re, im in _near_track_sums(x, y, z, ux, uy, uz, offsets, dt, omega, X0, Y0,
                                      L_screen):
        S = S + w[t] * dt * dt * (re * re + im * im).permute(2, 0, 1)
    return S.reshape(3, sinP.numel(), radius.numel(), omega.numel())


def near_cartesian_complex_torch(x, y, z, ux, uy, uz, w, offsets, dt, omega, radius, sinP,
                                 cosP, L_screen):
    """The coherent components [6][nPhi, nR, nOmega]: sqrt(w) dt Re A_x, Im A_x,
    Re A_y, ..., Im A_z summed over tracks (synchrad/kernel_nearfield.cl:216-326;
    no FormFactor)."""
    X0, Y0 = _screen(radius, sinP, cosP)
    D, O = X0.numel(), omega.numel()
    S = torch.zeros(6, D, O, dtype=torch.float64, device=x.device)
    for t, re, im in _near_track_sums(x, y, z, ux, uy, uz, offsets, dt, omega, X0, Y0,
                                      L_screen):
        S = S + torch.sqrt(w[t]) * dt * torch.stack([re, im], -1).permute(2, 3, 0, 1).reshape(6, D, O)
    return S.reshape(6, sinP.numel(), radius.numel(), omega.numel())
