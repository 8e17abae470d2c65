"""Post-processing of computed spectra as torch operations on the GPU.

``Utilities`` is the mixin that gives ``SynchRad`` the reference's
post-processing methods (``synchrad/utils.py:21-166``): the same method names,
arguments and results (numpy arrays), computed here as quadratures written as
weight vectors and applied with torch on the calculator's CUDA device (the CPU
only where no device exists, e.g. for a spectrum read back from a file on a
machine without one).

The physics is that of the reference: a spectrum S summed by the kernels
(``w dt^2 |A|^2`` per point, or the complex components) becomes the radiated
energy per unit frequency and solid angle (far field) or screen area (near
field) through the factor alpha / (2 pi)^2 (far) or alpha / (16 pi) (near);
the energy spectrum is its integral over the directions (trapezoid rule over
the midpoints of the theta axis with the sin(theta) Jacobian, far field) or
over the screen (trapezoid rule in R with the R Jacobian, near field), times
the phi step; the energy is the trapezoid integral of that over omega.  The
quadratures are formed once as weights (``_trapezoid_weights``,
``_direction_weights``) and contracted with the spectrum on the device, so
the same weights also give ``get_energy_weights`` for gradient-based use.

``get_spot_cartesian`` resamples the (theta or R, phi) map onto a Cartesian
grid with its own polar bilinear interpolation (see ``_polar_resample``),
not a scattered-data triangulation.  VTK export (tvtk) is not provided.
"""
from __future__ import annotations

import math

import numpy as np
import torch
from scipy import constants as _sc

# Photon energy in joules at a 1 um wavelength, h c / 1 um.
J_in_um = _sc.h * _sc.c / 1e-6
# Classical electron radius, e^2 / (4 pi eps0 m_e c^2), in metres.
r_e = _sc.e ** 2 / (4 * math.pi * _sc.epsilon_0 * _sc.m_e * _sc.c ** 2)
# Angular frequency of a 1 m wavelength (rad/s) and its photon energy in eV.
omega_1m = 2 * math.pi * _sc.c
energy_1m_eV = _sc.h * _sc.c / _sc.e


def _trapezoid_weights(x: torch.Tensor) -> torch.Tensor:
    """Weights q on the nodes x with sum(q * f) equal to the trapezoid
    integral of samples f over x (signed: a decreasing axis gives a negative
    integral, as numpy's trapezoid does).  Fewer than two nodes: zeros."""
    q = torch.zeros_like(x)
    if x.numel() > 1:
        half = 0.5 * (x[1:] - x[:-1])
        q[:-1] += half
        q[1:] += half
    return q


def _field_norm(mode: str) -> float:
    """alpha/(2 pi)^2 (far field) or alpha pi/4/(2 pi)^2 = alpha/(16 pi) (near)."""
    two_pi_sq = (2 * math.pi) ** 2
    if mode == "far":
        return _sc.alpha / two_pi_sq
    if mode == "near":
        return _sc.alpha * (math.pi / 4) / two_pi_sq
    raise ValueError(f"mode {mode!r}: post-processing is defined for 'far' and 'near'")


class Utilities:
    """Mixin of ``SynchRad``; reads ``self.Args``, ``self.Data['radiation']``
    and ``self.total_weight``."""

    # ------------------------------------------------------------------
    # device and inputs
    def _post_device(self) -> torch.device:
        dev = getattr(self, "device", None)
        if dev is not None and torch.device(dev).type == "cuda":
            return torch.device(dev)
        return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")

    def _axis(self, name: str, dev=None) -> torch.Tensor:
        a = np.asarray(self.Args[name], dtype=np.float64)
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev or self._post_device())

    def _snapshot(self, comp: str, iteration: int, dev) -> torch.Tensor:
        """The snapshot's spectrum, host layout (nOmega, nTheta|nR, nPhi):
        a comp's own array or, for 'total', the sum over the stored arrays
        (their squares for the coherent '*_complex' results); a component of a
        coherent result is returned complex, re + i im."""
        rad = self.Data["radiation"]

        def one(key):
            return torch.from_numpy(np.ascontiguousarray(
                np.asarray(rad[key][iteration], dtype=np.float64))).to(dev)

        coherent = self.Args["comp"].endswith("_complex")
        if comp != "total":
            if coherent:
                return torch.complex(one(comp + "re"), one(comp + "im"))
            return one(comp)
        parts = [one(k) for k in rad.keys()]
        if coherent:
            parts = [p * p for p in parts]
        out = parts[0].clone()
        for p in parts[1:]:
            out += p
        return out

    def _full(self, spect_filter=None, phot_num=False, lambda0_um=None,
              normalize_to_weights=False, comp="total", iteration=-1, dev=None):
        dev = dev or self._post_device()
        val = self._snapshot(comp, iteration, dev) * _field_norm(self.Args["mode"])
        if spect_filter is not None:
            val = val * torch.as_tensor(np.asarray(spect_filter), device=dev)
        if normalize_to_weights:
            val = val / float(self.total_weight)
        # photon number (per unit omega) takes precedence over the energy unit
        if phot_num:
            val = val / self._axis("omega", dev)[:, None, None]
        elif lambda0_um is not None:
            val = val * (J_in_um / lambda0_um)
        return val

    def _direction_weights(self, dev) -> torch.Tensor:
        """q over theta (far) or R (near) nodes with energy spectrum
        E(omega) = dphi * sum_phi sum_k q_k S(omega, k, phi).

        Far field: the integrand S sin(theta) is taken at the midpoints of the
        theta axis, the spectrum there being the mean of its two neighbours,
        and integrated by the trapezoid rule over the midpoints; each node gets
        half of the weight of each midpoint next to it.  Near field: the
        trapezoid rule in R of S R."""
        if self.Args["mode"] == "far":
            th = self._axis("theta", dev)
            mid = 0.5 * (th[1:] + th[:-1])
            per_mid = _trapezoid_weights(mid) * torch.sin(mid)
            q = torch.zeros_like(th)
            q[:-1] += 0.5 * per_mid
            q[1:] += 0.5 * per_mid
            return q
        r = self._axis("radius", dev)
        return _trapezoid_weights(r) * r

    # ------------------------------------------------------------------
    def get_full_spectrum(self, spect_filter=None, phot_num=False, lambda0_um=None,
                          normalize_to_weights=False, comp="total", iteration=-1):
        """Spectral energy density per unit frequency and solid angle (far) or
        screen area (near), host layout (nOmega, nTheta|nR, nPhi); with
        ``phot_num`` the photon number per unit frequency, with ``lambda0_um``
        in joules for that laser wavelength (synchrad/utils.py:23-73)."""
        return self._full(spect_filter, phot_num, lambda0_um, normalize_to_weights, comp,
                          iteration).cpu().numpy()

    def get_energy_spectrum(self, spect_filter=None, phot_num=False, lambda0_um=None,
                            **kw_args):
        """The full spectrum integrated over directions (far) or the screen
        (near): one value per omega (synchrad/utils.py:75-93)."""
        dev = self._post_device()
        val = self._full(spect_filter, phot_num, lambda0_um, dev=dev, **kw_args)
        q = self._direction_weights(dev).to(val.dtype)
        return (float(self.Args["dph"]) * torch.einsum("okp,k->o", val, q)).cpu().numpy()

    def get_energy(self, spect_filter=None, phot_num=False, lambda0_um=None, **kw_args):
        """The energy spectrum integrated over omega (synchrad/utils.py:95-102)."""
        dev = self._post_device()
        val = self._full(spect_filter, phot_num, lambda0_um, dev=dev, **kw_args)
        q_dir = self._direction_weights(dev).to(val.dtype)
        q_om = _trapezoid_weights(self._axis("omega", dev)).to(val.dtype)
        e = float(self.Args["dph"]) * torch.einsum("okp,k,o->", val, q_dir, q_om)
        return e.cpu().numpy()[()]

    def get_energy_weights(self, lambda0_um=None):
        """Weights q (host layout [nOmega, nTheta|nR, nPhi]) with
        ``get_energy(lambda0_um=...) == sum(q * S)`` for a 'total' spectrum S:
        the quadrature of get_energy_spectrum / get_energy written out, so that
        an energy loss can be differentiated through the spectrum (no
        counterpart in the reference)."""
        dev = self._post_device()
        c = _field_norm(self.Args["mode"]) * float(self.Args["dph"])
        if lambda0_um is not None:
            c = c * (J_in_um / lambda0_um)
        q = (c * _trapezoid_weights(self._axis("omega", dev))[:, None]
             * self._direction_weights(dev)[None, :])
        n_phi = len(self.Args["phi"])
        return q[:, :, None].expand(-1, -1, n_phi).contiguous().cpu().numpy()

    def get_spot(self, k0=None, spect_filter=None, phot_num=False, lambda0_um=None,
                 **kw_args):
        """The (theta or R, phi) map: the full spectrum integrated over omega
        (a single-frequency grid is scaled by its dw), or taken at one
        frequency picked from k0 (synchrad/utils.py:104-125)."""
        dev = self._post_device()
        val = self._full(spect_filter, phot_num, lambda0_um, dev=dev, **kw_args)
        omega = np.asarray(self.Args["omega"])
        if k0 is None:
            if val.shape[0] > 1:
                q = _trapezoid_weights(self._axis("omega", dev)).to(val.dtype)
                return torch.einsum("okp,o->kp", val, q).cpu().numpy()
            return (val[0].cpu().numpy() * np.asarray(self.Args["dw"]))
        # The frequency index: the count of axis values below k0, moved up by
        # one when the next value is strictly closer (an index past the axis
        # end raises IndexError).
        i = int(np.count_nonzero(omega < k0))
        if abs(omega[i + 1] - k0) < abs(omega[i] - k0):
            i += 1
        return val[i].cpu().numpy()

    def get_spot_cartesian(self, k0=None, th_part=1.0, bins=(200, 200), spect_filter=None,
                           phot_num=False, lambda0_um=None, **kw_args):
        """The spot of ``get_spot`` on a Cartesian grid of bins[0] x bins[1]
        points over [-m, m]^2, m = th_part x the largest theta (far) or R
        (near) node; returns (map, extent [-m, m, -m, m]).  Points outside the
        sampled (radius, phi) domain are 0 (synchrad/utils.py:127-152
        resamples with a triangulation instead; see _polar_resample)."""
        spot = self.get_spot(k0=k0, spect_filter=spect_filter, phot_num=phot_num,
                             lambda0_um=lambda0_um, **kw_args)
        mode = self.Args["mode"]
        if mode not in ("far", "near"):
            raise ValueError("get_spot_cartesian is defined for the 'far' and 'near' modes")
        dev = self._post_device()
        radial = self._axis("theta" if mode == "far" else "radius", dev)
        phi = self._axis("phi", dev)
        m = th_part * float(radial.max())
        xs = torch.linspace(-m, m, int(bins[0]), dtype=torch.float64, device=dev)
        ys = torch.linspace(-m, m, int(bins[1]), dtype=torch.float64, device=dev)
        out = _polar_resample(torch.as_tensor(spot, device=dev), radial, phi, xs, ys)
        return out.cpu().numpy(), np.array([-m, m, -m, m])

    def get_spectral_axis(self):
        """The frequency axis of the spectra (synchrad/utils.py:154-166)."""
        return self.Args["omega"]


def _polar_resample(spot: torch.Tensor, radial: torch.Tensor, phi: torch.Tensor,
                    xs: torch.Tensor, ys: torch.Tensor) -> torch.Tensor:
    """Bilinear interpolation in (radius, phi) of ``spot[k, j]`` (radius node k,
    phi node j) at the Cartesian points (xs[a], ys[b]); returns [len(xs), len(ys)].

    A point's radius and angle locate its cell between two radius nodes and
    two phi nodes; the value is bilinear in the radius and angle fractions, so
    every node is reproduced exactly and values along each ray and ring are
    linear between nodes.  A phi axis that closes the circle (n_phi steps of
    dphi make 2 pi) interpolates across the seam; an open one leaves angles
    outside [phi_0, phi_last] at 0, as it does radii below r_0.  The outer
    boundary is the polygon through the outermost ring's nodes (the straight
    chord between neighbouring nodes, not the arc), the convex hull of the
    samples: points between chord and arc are 0.

    On a polar grid each cell's four nodes lie on one circle, so a Delaunay
    triangulation of them (the reference's griddata) has no unique diagonal
    and its values inside a cell depend on the library's tie-breaking; the
    two agree at the nodes and differ inside cells by the interpolation error.
    """
    nr, nphi = int(radial.numel()), int(phi.numel())
    if nr < 2 or nphi < 2:
        raise ValueError("resampling needs at least two radius and two phi nodes")
    X, Y = torch.meshgrid(xs, ys, indexing="ij")
    rad = torch.hypot(X, Y)
    dphi = float(phi[1] - phi[0])
    two_pi = 2 * math.pi
    closed = abs(nphi * dphi - two_pi) <= 1e-9 * two_pi
    ang = torch.remainder(torch.atan2(Y, X) - float(phi[0]), two_pi)
    # radius cell k: radial[k] <= rad <= radial[k + 1]
    k = (torch.searchsorted(radial.contiguous(), rad.reshape(-1), right=True) - 1)
    k = k.clamp(0, nr - 2).reshape(rad.shape)
    r0, r1 = radial[k], radial[k + 1]
    s = ((rad - r0) / (r1 - r0)).clamp(0.0, 1.0)
    inside = (rad >= radial[0]) & (rad <= radial[-1])
    # phi cell j: the angle measured from phi_0 in steps of dphi
    u = ang / dphi
    j = torch.floor(u).long()
    if closed:
        j = j.clamp(0, nphi - 1)
        j1 = torch.remainder(j + 1, nphi)
    else:
        inside &= u <= nphi - 1
        j = j.clamp(0, nphi - 2)
        j1 = j + 1
    t = (u - j.to(u.dtype)).clamp(0.0, 1.0)
    # inside the chord of the outer ring between phi nodes j and j + 1
    half = 0.5 * dphi
    chord = float(radial[-1]) * math.cos(half) / torch.cos((t - 0.5) * dphi)
    inside &= rad <= chord * (1.0 + 1e-12)
    v00, v10 = spot[k, j], spot[k + 1, j]
    v01, v11 = spot[k, j1], spot[k + 1, j1]
    val = ((1 - s) * (1 - t) * v00 + s * (1 - t) * v10 + (1 - s) * t * v01 + s * t * v11)
    return torch.where(inside, val, torch.zeros_like(val))
