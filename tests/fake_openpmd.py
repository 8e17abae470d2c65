"""Stand-ins for openPMD-viewer's ``OpenPMDTimeSeries`` and ``ParticleTracker``
(neither installed here) with the members the track converters use, over a
seeded synthetic particle history, and a synthetic VSIM tracks array.

``scenario()`` builds the particle data: 12 particles over 40 iterations with
absences (NaN) that split, delay, end and shorten tracks, and one iteration
whose arrays miss a particle (the converters then treat the whole iteration as
absent).  Particle ids are their indices.
"""
from __future__ import annotations

import numpy as np

VARS = ("x", "y", "z", "ux", "uy", "uz", "w", "id")


class FakeSeries:
    def __init__(self, data, iterations, t, short_iterations=()):
        self.data = data
        self.iterations = np.asarray(iterations)
        self.t = np.asarray(t, dtype=np.float64)
        self.short = set(int(i) for i in short_iterations)

    def get_particle(self, var_list=None, select=None, species=None, iteration=None):
        k = int(np.flatnonzero(self.iterations == iteration)[0])
        idx = np.asarray(select.selected_pid, dtype=np.int64)
        out = [np.array(self.data[v][k, idx]) for v in var_list]
        if int(iteration) in self.short:
            out = [o[:-1] for o in out]
        return out

    def iterate(self, called_method, **kwargs):
        per_it = [called_method(iteration=it, **kwargs) for it in self.iterations]
        return tuple([r[i] for r in per_it] for i in range(len(per_it[0])))


class FakeTracker:
    def __init__(self, ts, species=None, iteration=None, select=None,
                 preserve_particle_index=False):
        self.species = species
        self.selected_pid = np.array(select, dtype=np.int64)
        self.N_selected = int(self.selected_pid.size)


def scenario(gaps=True):
    """(series, tracker over every particle)."""
    rng = np.random.default_rng(17)
    n_it, n_p = 40, 12
    iterations = 10 * np.arange(n_it)
    t = iterations * 2.5e-15
    k = np.arange(n_it)[:, None]
    phase = rng.uniform(0, 2 * np.pi, n_p)[None, :]
    data = {
        "x": 1e-6 * np.sin(0.3 * k + phase),
        "y": 5e-7 * np.cos(0.2 * k + phase),
        "z": 1e-6 * k + 1e-7 * phase,
        "ux": 0.1 * np.cos(0.3 * k + phase),
        "uy": 0.05 * np.sin(0.2 * k + phase),
        "uz": 100.0 + 0.01 * k + phase,
        "w": np.broadcast_to(rng.uniform(0.5, 2.0, n_p)[None, :], (n_it, n_p)).copy(),
        "id": np.broadcast_to(np.arange(n_p, dtype=np.float64)[None, :], (n_it, n_p)).copy(),
    }
    short = ()
    if gaps:
        absent = np.zeros((n_it, n_p), dtype=bool)
        absent[10:16, 2] = True      # a gap: two pieces
        absent[:8, 5] = True         # appears late
        absent[30:, 7] = True        # leaves early
        absent[:, 9] = True
        absent[12:17, 9] = False     # present for 5 iterations only
        absent[3:5, 11] = True
        absent[25:27, 11] = True     # two gaps: three pieces
        for v in data:
            data[v][absent] = np.nan
        short = (int(iterations[20]),)
    ts = FakeSeries(data, iterations, t, short)
    return ts, FakeTracker(ts, species="electrons", select=np.arange(n_p))


def vsim_tracks():
    """[Nt, Np, 6] of z, y, x, uz, uy, ux (SI): x <= 0 marks steps outside the
    box (particles entering late; one inside for 5 steps only)."""
    rng = np.random.default_rng(23)
    n_t, n_p = 30, 10
    k = np.arange(n_t)[:, None]
    ph = rng.uniform(0, 2 * np.pi, n_p)[None, :]
    x = 2e-6 + 1e-6 * np.sin(0.4 * k + ph)
    enter = np.array([0, 0, 3, 7, 0, 12, 25, 1, 0, 5])
    x[k < enter[None, :]] = -1.0
    z = 1e-6 * k + 1e-7 * ph
    y = 1e-6 * np.cos(0.3 * k + ph)
    c0 = 299792458.0
    ux = c0 * 0.1 * np.cos(0.4 * k + ph)
    uy = c0 * 0.05 * np.sin(0.3 * k + ph)
    uz = c0 * (50.0 + ph + 0 * k)
    return np.stack([z, y, x, uz, uy, ux], -1)
