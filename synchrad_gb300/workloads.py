"""Seeded synthetic particle tracks and grids for the benchmark workloads.

Units follow the reference: c = 1, lengths in a user unit (the undulator or
betatron period), ``timeStep`` = c*dt in that unit, spectral grid omega in
1/unit (the device multiplies by 2*pi, ``synchrad/calc.py:493-495``).

Far-field tracks are staggered like the reference tutorials and tests
(positions at t_s, momenta at t_s - dt/2, ``tests/test_undulator_analytic.py:27-50``);
near-field tracks are unstaggered (``synchrad/kernel_nearfield.cl:79-82``
uses u at the same step as x).

One "micrometre-equivalent" is 1e-6 m with the undulator period pinned to
15 mm (so 2 um = 1.333e-4 periods); for betatron tracks the unit is a 1 mm
betatron period (1 um = 1e-3 units).

Every generator returns tracks in the reference's list format
``[x, y, z, ux, uy, uz, w, it_start]``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

UM_PER_UNDULATOR_PERIOD = 15e-3 / 1e-6     # 15 mm period
UM_PER_BETATRON_PERIOD = 1e-3 / 1e-6       # 1 mm betatron period


def _envelope(z, n_periods, ramp):
    """Linear entry/exit ramps of `ramp` periods around a flat top [0, n_periods]."""
    up = np.clip((z + ramp) / ramp, 0.0, 1.0)
    down = np.clip((n_periods + ramp - z) / ramp, 0.0, 1.0)
    return up * down


def undulator_track(gamma, K, n_periods, dt, n_steps=None, ramp=1.0, x0=0.0,
                    y0=0.0, xp=0.0, yp=0.0, helical=False, stagger=True,
                    weight=1.0, dtype=np.float64):
    """Analytic planar (or helical) undulator track along z, period = 1.

    The construction follows the reference's analytic test: z = v t with the
    mean drift velocity, u_x = K sin(2 pi z) under the ramp envelope (a half
    step earlier when ``stagger``), u_z from gamma, x from the running sum of
    u_x/gamma.  ``x0, y0`` offset and ``xp, yp`` tilt the whole track.
    """
    if n_steps is None:
        n_steps = int(round((n_periods + 2 * ramp) / dt))
    t = -ramp + dt * np.arange(n_steps, dtype=np.float64)
    k_eff = K if not helical else K * np.sqrt(2.0)
    gz = gamma / np.sqrt(1.0 + k_eff ** 2 / 2)
    vb = np.sqrt(1.0 - gz ** -2)
    z = vb * t
    zs = z - 0.5 * dt if stagger else z
    env = _envelope(zs, n_periods, ramp)
    ux = K * env * np.sin(2 * np.pi * zs)
    uy = K * env * np.cos(2 * np.pi * zs) if helical else np.zeros_like(ux)
    uz = np.sqrt(gamma ** 2 - 1.0 - ux ** 2 - uy ** 2)
    if stagger:
        x = ux[0] / gamma * dt / 2 + np.cumsum(ux / gamma) * dt
        y = uy[0] / gamma * dt / 2 + np.cumsum(uy / gamma) * dt
    else:
        x = np.concatenate(([0.0], np.cumsum(ux[:-1] / gamma) * dt))
        y = np.concatenate(([0.0], np.cumsum(uy[:-1] / gamma) * dt))
    x = x + x0 + xp * z
    y = y + y0 + yp * z
    ux = ux + xp * uz
    uy = uy + yp * uz
    uz = np.sqrt(gamma ** 2 - 1.0 - ux ** 2 - uy ** 2)
    arrs = [np.ascontiguousarray(a, dtype=dtype) for a in (x, y, z, ux, uy, uz)]
    return arrs + [float(weight), 0]


def betatron_track(gamma, amp_x, phase_x, n_steps, dt, amp_y=0.0, phase_y=0.0,
                   weight=1.0, dtype=np.float64):
    """Betatron-like track: x = A sin(2 pi z + psi), period 1, leapfrog momenta."""
    t = dt * np.arange(n_steps + 1, dtype=np.float64)
    k_b = 2 * np.pi * gamma * max(amp_x, amp_y)
    gz = gamma / np.sqrt(1.0 + k_b ** 2 / 2)
    z = np.sqrt(1.0 - gz ** -2) * t
    x = amp_x * np.sin(2 * np.pi * z + phase_x)
    y = amp_y * np.sin(2 * np.pi * z + phase_y)
    ux = gamma * np.diff(x) / dt
    uy = gamma * np.diff(y) / dt
    x, y, z = x[:-1], y[:-1], z[:-1]
    uz = np.sqrt(np.maximum(gamma ** 2 - 1.0 - ux ** 2 - uy ** 2, 1.0))
    arrs = [np.ascontiguousarray(a, dtype=dtype) for a in (x, y, z, ux, uy, uz)]
    return arrs + [float(weight), 0]


@dataclass
class Workload:
    name: str
    args: dict                       # SynchRad constructor Args
    tracks: list                     # reference track lists
    time_step: float
    comp: str = "total"
    L_screen: float | None = None
    notes: dict = field(default_factory=dict)

    @property
    def n_points(self) -> int:
        return int(np.prod(self.args["grid"][-1]))

    @property
    def pt_steps(self) -> int:
        """Spectral points x sum over tracks of (steps - 1): the metric's unit."""
        return self.n_points * int(sum(max(len(t[0]) - 1, 0) for t in self.tracks))


def fundamental(gamma, K):
    """On-axis undulator fundamental 2 gamma^2/(1 + K^2/2), in 1/period."""
    return 2 * gamma ** 2 / (1 + K ** 2 / 2)


def c1_single_undulator(grid=(256, 32, 32)) -> Workload:
    """1 electron, gamma 100, K 0.1, 20 periods + 1-period ramps, 64 steps/period."""
    g, K = 100.0, 0.1
    dt = 1.0 / 64
    tr = undulator_track(g, K, 20, dt, ramp=1.0)
    w1 = fundamental(g, K)
    args = {"grid": [(0.5 * w1, 1.5 * w1), (0.0, 1.0 / g), (0.0, 2 * np.pi), tuple(grid)],
            "dtype": "double"}
    return Workload("far_fp64_1e_g100_K0.1_1408steps_256x32x32", args, [tr], dt)


def c2_far_mixed(n_tracks=1024, n_steps=4000, grid=(512, 64, 64), seed=0,
                 n_periods=60) -> Workload:
    """1024 electrons, gamma ~ N(400, 1%), K = 1, offsets N(0, 2 um-eq),
    angles N(0, 0.05/gamma), 4000 steps, w ~ U[0.5, 1.5]; first three harmonics."""
    rng = np.random.default_rng(seed)
    g0, K = 400.0, 1.0
    dt = (n_periods + 2.0) / n_steps
    sig_x = 2.0 / UM_PER_UNDULATOR_PERIOD
    tracks = []
    for _ in range(n_tracks):
        g = g0 * (1 + 0.01 * rng.standard_normal())
        x0, y0 = sig_x * rng.standard_normal(2)
        xp, yp = (0.05 / g0) * rng.standard_normal(2)
        w = rng.uniform(0.5, 1.5)
        tracks.append(undulator_track(g, K, n_periods, dt, n_steps=n_steps, x0=x0,
                                      y0=y0, xp=xp, yp=yp, weight=w))
    w1 = fundamental(g0, K)
    args = {"grid": [(0.5 * w1, 3.5 * w1), (0.0, 2.0 / g0), (0.0, 2 * np.pi), tuple(grid)],
            "dtype": "mixed"}
    return Workload(f"far_mixed_{n_tracks}e_g400_K1_{n_steps}steps_"
                    f"{grid[0]}x{grid[1]}x{grid[2]}", args, tracks, dt,
                    notes={"seed": seed})


def c3_betatron_ragged(n_tracks=8192, grid=(256, 48, 48), seed=0,
                       steps_range=(500, 20000)) -> Workload:
    """8192 betatron-like tracks, gamma ~ U(200, 800), amplitude ~ U(0.5, 3) um-eq,
    random phase, steps ~ U{500..20000}, FP32 positions and momenta, random weights."""
    rng = np.random.default_rng(seed)
    dt = 1.0 / 64
    tracks = []
    for _ in range(n_tracks):
        g = rng.uniform(200, 800)
        ax = rng.uniform(0.5, 3.0) / UM_PER_BETATRON_PERIOD
        ay = 0.3 * rng.uniform(0.5, 3.0) / UM_PER_BETATRON_PERIOD
        ph = rng.uniform(0, 2 * np.pi, 2)
        n = int(rng.integers(steps_range[0], steps_range[1] + 1))
        tracks.append(betatron_track(g, ax, ph[0], n, dt, amp_y=ay, phase_y=ph[1],
                                     weight=rng.uniform(0.5, 1.5), dtype=np.float32))
    args = {"grid": [(2e3, 2e5), (0.0, 0.025), (0.0, 2 * np.pi), tuple(grid)],
            "dtype": "mixed"}
    return Workload(f"far_mixed_ragged_{n_tracks}betatron_{grid[0]}x{grid[1]}x{grid[2]}",
                    args, tracks, dt, notes={"seed": seed})


def c4_adjoint(n_tracks=256, n_steps=2000, grid=(128, 32, 32), seed=0,
               n_periods=30) -> Workload:
    """256 electrons, K = 0.5, 2000 steps; spectrum 128 x 32 x 32."""
    rng = np.random.default_rng(seed)
    g0, K = 200.0, 0.5
    dt = (n_periods + 2.0) / n_steps
    tracks = []
    for _ in range(n_tracks):
        g = g0 * (1 + 0.005 * rng.standard_normal())
        x0, y0 = (1.0 / UM_PER_UNDULATOR_PERIOD) * rng.standard_normal(2)
        tracks.append(undulator_track(g, K, n_periods, dt, n_steps=n_steps, x0=x0,
                                      y0=y0, weight=rng.uniform(0.5, 1.5)))
    w1 = fundamental(g0, K)
    args = {"grid": [(0.5 * w1, 1.5 * w1), (0.0, 1.5 / g0), (0.0, 2 * np.pi), tuple(grid)],
            "dtype": "mixed"}
    return Workload(f"far_adjoint_{n_tracks}e_K0.5_{n_steps}steps", args, tracks, dt,
                    notes={"seed": seed})


def perturbed_tracks(tracks, rel=1e-3, seed=1):
    """Copies of ``tracks`` with x, y scaled by (1 + rel N(0,1)) and the
    momenta by (1 + rel N(0,1)) (gamma changes by about the same relative
    amount), one draw per track: the target tracks of the adjoint workload."""
    rng = np.random.default_rng(seed)
    out = []
    for t in tracks:
        fx, fu = 1.0 + rel * rng.standard_normal(2)
        c = [np.asarray(a).copy() for a in t[:6]]
        c[0] *= fx
        c[1] *= fx
        for k in (3, 4, 5):
            c[k] *= fu
        out.append(c + list(t[6:]))
    return out


def c5_near_helical(n_tracks=2048, n_steps=8000, grid=(256, 64, 64), seed=0,
                    n_periods=50) -> Workload:
    """2048 electrons in a helical undulator, gamma ~ N(300, 2%), 8000 steps,
    screen at 20 undulator lengths; grid 256 omega x 64 R x 64 phi."""
    rng = np.random.default_rng(seed)
    g0, K = 300.0, 0.5
    dt = (n_periods + 2.0) / n_steps
    tracks = []
    for _ in range(n_tracks):
        g = g0 * (1 + 0.02 * rng.standard_normal())
        x0, y0 = (2.0 / UM_PER_UNDULATOR_PERIOD) * rng.standard_normal(2)
        tracks.append(undulator_track(g, K, n_periods, dt, n_steps=n_steps, x0=x0,
                                      y0=y0, helical=True, stagger=False,
                                      weight=rng.uniform(0.5, 1.5)))
    L = 20.0 * n_periods
    w1 = 2 * g0 ** 2 / (1 + K ** 2)
    args = {"grid": [(0.5 * w1, 1.5 * w1), (0.0, 1.5 * L / g0), (0.0, 2 * np.pi),
                     tuple(grid)],
            "mode": "near", "dtype": "mixed"}
    return Workload(f"near_mixed_{n_tracks}e_helical_{n_steps}steps", args, tracks, dt,
                    L_screen=L, notes={"seed": seed})


def analytic_undulator_tracks(n_particles=24, K=0.1, n_periods=50, g0=100.0,
                              steps_per_period=32, seed=0, stagger=True):
    """Tracks of the reference's analytic undulator checks (energy spread 1e-4),
    with a fixed seed.  Returns (tracks, dt, k_res)."""
    rng = np.random.default_rng(seed)
    dt = 1.0 / steps_per_period
    n_steps = int((n_periods + 2) / dt) + 1
    t = np.linspace(-1, n_periods + 1, n_steps)
    gg = g0 / (1.0 + K ** 2 / 2) ** 0.5
    k_res = 2 * gg ** 2
    tracks = []
    for g in g0 + 1e-4 * g0 * rng.standard_normal(n_particles):
        ggp = g / (1.0 + K ** 2 / 2) ** 0.5
        z = (1.0 - ggp ** -2) ** 0.5 * t
        zs = z - 0.5 * dt if stagger else z
        env = (((zs > 0) * (zs < 1.5) * zs / 1.5 + (zs > 1.5))
               * ((zs > n_periods - 1.5) * (zs < n_periods) * (n_periods - zs) / 1.5
                  + (zs < n_periods - 1.5)))
        ux = K * np.sin(2 * np.pi * zs) * env
        uz = (g0 ** 2 - 1 - ux ** 2) ** 0.5
        x = ux[0] / g * dt / 2 + np.cumsum(ux / g) * dt
        zeros = np.zeros_like(t)
        tracks.append([x, zeros.copy(), z, ux, zeros.copy(), uz, 1.0, 0])
    return tracks, dt, k_res
