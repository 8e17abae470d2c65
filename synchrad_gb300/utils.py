"""Post-processing of computed spectra: the reference's ``Utilities`` mixin.

Same methods, arguments and normalisation as ``synchrad/utils.py:21-166``:
physical constants alpha/(4 pi^2) (far field) or alpha pi/4/(2 pi)^2 (near
field), theta (far) or R (near) integration, energy integrals and spot maps.
This is host numpy work on already-computed spectra; VTK export (tvtk) is not
provided.
"""
from __future__ import annotations

import numpy as np
from scipy.constants import c, e, epsilon_0, hbar, m_e
from scipy.constants import alpha as alpha_fs

J_in_um = 2e6 * np.pi * hbar * c
r_e = e ** 2 / (4 * np.pi * epsilon_0 * m_e * c ** 2)
omega_1m = 2 * np.pi * c
energy_1m_eV = omega_1m * hbar / e

_trapz = getattr(np, "trapezoid", None) or getattr(np, "trapz")


class Utilities:
    """Mixin of SynchRad; expects ``self.Args``, ``self.Data['radiation']``,
    ``self.total_weight``."""

    def get_full_spectrum(self, spect_filter=None, phot_num=False, lambda0_um=None,
                          normalize_to_weights=False, comp="total", iteration=-1):
        """synchrad/utils.py:23-73."""
        keys = self.Data["radiation"].keys()
        val = 0.0
        if self.Args["comp"].split("_")[-1] == "complex":
            if comp == "total":
                for key in keys:
                    val += self.Data["radiation"][key][iteration].astype(np.double) ** 2
            else:
                val = (self.Data["radiation"][comp + "re"][iteration].astype(np.complex128)
                       + 1.0j * self.Data["radiation"][comp + "im"][iteration]
                       .astype(np.complex128))
        else:
            if comp == "total":
                for key in keys:
                    val += self.Data["radiation"][key][iteration].astype(np.double)
            else:
                val += self.Data["radiation"][comp][iteration].astype(np.double)

        if self.Args["mode"] == "far":
            val = alpha_fs / (4 * np.pi ** 2) * val
        elif self.Args["mode"] == "near":
            val = alpha_fs * np.pi / 4 * val
            val /= (2 * np.pi) ** 2

        if spect_filter is not None:
            val *= spect_filter
        if normalize_to_weights:
            val /= self.total_weight
        if phot_num:
            ax = self.Args["omega"]
            val /= ax[:, None, None]
        elif lambda0_um is not None:
            val *= J_in_um / lambda0_um
        return val

    def get_energy_spectrum(self, spect_filter=None, phot_num=False, lambda0_um=None,
                            **kw_args):
        """synchrad/utils.py:75-93: integrate over theta (far) or R (near) and phi."""
        val = self.get_full_spectrum(spect_filter=spect_filter, phot_num=phot_num,
                                     lambda0_um=lambda0_um, **kw_args)
        if self.Args["mode"] == "far":
            theta_loc = 0.5 * (self.Args["theta"][1:] + self.Args["theta"][:-1])
            val_loc = 0.5 * (val[:, 1:, :] + val[:, :-1, :])
            int_theta = _trapz(val_loc * np.sin(theta_loc)[None, :, None], theta_loc, axis=1)
            val = self.Args["dph"] * int_theta.sum(-1)
        elif self.Args["mode"] == "near":
            r_loc = self.Args["radius"]
            int_r = _trapz(val * r_loc[None, :, None], r_loc, axis=1)
            val = self.Args["dph"] * int_r.sum(-1)
        return val

    def get_energy(self, spect_filter=None, phot_num=False, lambda0_um=None, **kw_args):
        """synchrad/utils.py:95-102: integrate the energy spectrum over omega."""
        val = self.get_energy_spectrum(spect_filter=spect_filter, phot_num=phot_num,
                                       lambda0_um=lambda0_um, **kw_args)
        return _trapz(val, self.Args["omega"])

    def get_energy_weights(self, lambda0_um=None):
        """Weights q (host layout [nOmega, nTheta|nR, nPhi]) with
        ``get_energy(lambda0_um=...) == sum(q * S)`` for a 'total' spectrum S:
        the quadrature of get_energy_spectrum / get_energy written out, so that
        an energy loss can be differentiated through the spectrum (no
        counterpart in the reference)."""
        def trapz_w(x):
            x = np.asarray(x, dtype=np.double)
            w = np.zeros_like(x)
            if x.size > 1:
                d = np.diff(x)
                w[:-1] += 0.5 * d
                w[1:] += 0.5 * d
            return w

        if self.Args["mode"] == "far":
            c = alpha_fs / (4 * np.pi ** 2)
            th = np.asarray(self.Args["theta"], dtype=np.double)
            th_loc = 0.5 * (th[1:] + th[:-1])
            a = trapz_w(th_loc) * np.sin(th_loc)
            ang = np.zeros_like(th)
            ang[:-1] += 0.5 * a
            ang[1:] += 0.5 * a
        elif self.Args["mode"] == "near":
            c = alpha_fs * np.pi / 4 / (2 * np.pi) ** 2
            r = np.asarray(self.Args["radius"], dtype=np.double)
            ang = trapz_w(r) * r
        else:
            raise ValueError("energy weights are defined for the 'far' and 'near' modes")
        if lambda0_um is not None:
            c = c * J_in_um / lambda0_um
        w_om = trapz_w(self.Args["omega"])
        n_phi = len(self.Args["phi"]) if "phi" in self.Args else None
        q = c * self.Args["dph"] * w_om[:, None] * ang[None, :]
        return np.repeat(q[:, :, None], n_phi if n_phi else 1, axis=2)

    def get_spot(self, k0=None, spect_filter=None, phot_num=False, lambda0_um=None,
                 **kw_args):
        """synchrad/utils.py:104-125: angular (or screen) map, integrated over
        omega or taken at the frequency nearest to ``k0``."""
        val = self.get_full_spectrum(spect_filter=spect_filter, phot_num=phot_num,
                                     lambda0_um=lambda0_um, **kw_args)
        if k0 is None:
            if val.shape[0] > 1:
                val = _trapz(val, self.Args["omega"], axis=0)
            else:
                val = val[0] * self.Args["dw"]
        else:
            ax = self.Args["omega"]
            indx = (ax < k0).sum()
            if np.abs(self.Args["omega"][indx + 1] - k0) < np.abs(self.Args["omega"][indx] - k0):
                indx += 1
            val = val[indx]
        return val

    def get_spot_cartesian(self, k0=None, th_part=1.0, bins=(200, 200), spect_filter=None,
                           phot_num=False, lambda0_um=None, **kw_args):
        """synchrad/utils.py:127-152: the spot resampled on a Cartesian grid."""
        from scipy.interpolate import griddata

        val = self.get_spot(spect_filter=spect_filter, k0=k0, phot_num=phot_num,
                            lambda0_um=lambda0_um, **kw_args)
        if self.Args["mode"] == "far":
            th, ph = self.Args["theta"], self.Args["phi"]
        else:
            th, ph = self.Args["radius"], self.Args["phi"]
        ph, th = np.meshgrid(ph, th)
        coord = ((th * np.cos(ph)).flatten(), (th * np.sin(ph)).flatten())
        th_max = th_part * th.max()
        new_coord = np.mgrid[-th_max:th_max:bins[0] * 1j, -th_max:th_max:bins[1] * 1j]
        val = griddata(coord, val.flatten(), (new_coord[0].flatten(), new_coord[1].flatten()),
                       fill_value=0.0, method="linear").reshape(new_coord[0].shape)
        ext = np.array([-th_max, th_max, -th_max, th_max])
        return val, ext

    def get_spectral_axis(self):
        """synchrad/utils.py:154-166."""
        return self.Args["omega"]
