"""Track converters: particle data of PIC codes -> SynchRad track files.

The same functions, arguments and file layout as ``synchrad/converters.py``:
a track file holds ``tracks/<i>/{x,y,z,ux,uy,uz,w,it_start}`` and
``misc/{cdt, N_particles, it_range, propagation_direction}`` (``tracksFromOPMD``
also ``misc/cdt_array``), which ``SynchRad.calculate_spectrum(file_tracks=...)``
reads (``synchrad/calc.py:186-219``).  Host-side I/O with numpy and h5py; the
per-particle loops of the reference are array operations here.

* ``tracksFromOPMD`` (synchrad/converters.py:19-128): openPMD-viewer
  ``OpenPMDTimeSeries`` + ``ParticleTracker`` -> track file;
* ``tracksFromOPMD_old`` (:130-228): the earlier reader, to a file or to a
  list of tracks;
* ``tracksFromVSIM`` (:230-293): a VSIM ``tracks`` dataset [Nt, Np, 6] ->
  track file;
* ``split_track_by_nans`` (:295-352), ``record_particles_step`` (:354-374),
  ``record_particles_first`` (:376-393): the helpers.
"""
from __future__ import annotations

import numpy as np
from scipy.constants import c

_COORDS = ("x", "y", "z", "ux", "uy", "uz")


def _h5():
    import h5py
    return h5py


def split_track_by_nans(x, y, z, ux, uy, uz, w):
    """Pieces of a particle's history between the iterations where ``w`` is NaN.

    Returns ``[x, y, z, ux, uy, uz, w0, it0]`` per non-empty piece, ``w0`` the
    weight and ``it0`` the iteration index at its first step."""
    w = np.asarray(w)
    present = ~np.isnan(w)
    edges = np.diff(np.concatenate([[False], present, [False]]).astype(np.int8))
    starts = np.flatnonzero(edges == 1)
    ends = np.flatnonzero(edges == -1)
    cols = [np.asarray(v) for v in (x, y, z, ux, uy, uz)]
    pieces = []
    for a, b in zip(starts, ends):
        sl = slice(a, b)
        pieces.append([np.array(v[sl]) for v in cols] + [w[a], a])
    return pieces


def record_particles_first(tracks, nsteps, it, it_start, x, y, z, ux, uy, uz, id, Np_select):
    """Appends iteration ``it`` of the first ``Np_select`` particles to
    ``tracks[step, particle, 7]`` (NaN positions are absent particles)."""
    return record_particles_step(tracks, nsteps, it, it_start, x, y, z, ux, uy, uz, id,
                                 Np_select, 1)


def record_particles_step(tracks, nsteps, it, it_start, x, y, z, ux, uy, uz, id,
                          Np_select, dNp):
    """Appends iteration ``it`` of every ``dNp``-th particle (``Np_select`` of
    them) to ``tracks[step, particle, 7]``; a particle's first recorded
    iteration goes to ``it_start`` (0 meaning unset, as in the reference)."""
    sel = np.arange(Np_select) * dNp
    xs = np.asarray(x)[sel]
    ok = ~np.isnan(xs)
    ip = np.flatnonzero(ok)
    unset = ip[it_start[ip] == 0]
    it_start[unset] = it
    rows = np.stack([np.asarray(v)[sel][ok] for v in (x, y, z, ux, uy, uz, id)], -1)
    tracks[nsteps[ip], ip, :] = rows
    nsteps[ip] += 1
    return tracks, nsteps, it_start


def tracksFromOPMD(ts, pt, ref_iteration, fname="./tracks.h5", Np_select=None, dNp=1,
                   sample_selection="random", Nit_min=None, Nit_max=None, z_is_xi=False,
                   shortest_track=8):
    """Tracks of the particles selected by ``pt`` (an openPMD-viewer
    ``ParticleTracker`` on ``ts``) written to ``fname``.

    ``Np_select`` particles are drawn from the tracker's selection
    (``np.random.choice``, with replacement, for 'random'; the first ones for
    'sequential'), then every ``dNp``-th is kept; each particle's history is
    cut into pieces where it is absent (NaN), and pieces longer than
    ``shortest_track`` steps become tracks.  ``z_is_xi`` adds c t to z (the
    co-moving coordinate back to the lab frame) with t of the piece's own
    iterations; the reference adds the whole (Nit-filtered) time axis, which
    agrees for a piece that spans every iteration and raises otherwise."""
    all_pid = pt.selected_pid.copy()
    selected = all_pid
    if Np_select is not None:
        if all_pid.size < Np_select:
            Np_select = all_pid.size
            print(f"Selected sample of {Np_select} tracks it too large. ",
                  f"Only {all_pid.size} tracks are available in ParticleTracker")
        if sample_selection == "random":
            selected = np.random.choice(all_pid, size=Np_select)
        elif sample_selection == "sequential":
            selected = all_pid[:Np_select]
        else:
            print(f"Selected sampling method '{sample_selection}' is ", "not available.")
    if dNp > 1:
        selected = selected[::dNp]
    pt.__init__(ts, species=pt.species, iteration=ref_iteration, select=selected,
                preserve_particle_index=True)

    iterations = ts.iterations.copy()
    keep = np.ones(iterations.size, dtype=bool)
    if Nit_min is not None:
        keep &= iterations >= Nit_min
    if Nit_max is not None:
        keep &= iterations <= Nit_max
    t_all = ts.t.copy()
    t = t_all[keep]
    cdt = (t[1] - t[0]) * c
    cdt_array = (t[1:] - t[:-1]) * c

    names = list(_COORDS) + ["w"]
    per_iteration = ts.iterate(ts.get_particle, select=pt, var_list=names, species=pt.species)
    n_sel = pt.N_selected
    data = {}
    for name, series in zip(names, per_iteration):
        # iterations whose arrays do not cover the selection count as absent
        rows = [np.asarray(v) if len(v) == n_sel else np.full(n_sel, np.nan)
                for v in series]
        data[name] = np.array(rows, order="F").T          # [particle, iteration]
    incomplete = [len(v) != n_sel for v in per_iteration[0]]
    for name in names:
        data[name][:, incomplete] = np.nan

    h5 = _h5()
    f = h5.File(fname, mode="w")
    n_tr, it_lo, it_hi = 0, np.inf, 0
    for ip in range(n_sel):
        pieces = split_track_by_nans(*(data[k][ip] for k in names))
        for px, py, pz, pux, puy, puz, pw, p0 in pieces:
            n = px.size
            if n <= shortest_track:
                continue
            g = f"tracks/{n_tr:d}/"
            f[g + "x"] = px
            f[g + "y"] = py
            f[g + "z"] = pz + c * t_all[p0:p0 + n] if z_is_xi else pz
            f[g + "ux"] = pux
            f[g + "uy"] = puy
            f[g + "uz"] = puz
            f[g + "w"] = pw
            f[g + "it_start"] = p0
            it_hi = max(it_hi, p0 + n)
            it_lo = min(it_lo, p0)
            n_tr += 1
    f["misc/cdt"] = cdt
    f["misc/cdt_array"] = cdt_array
    f["misc/N_particles"] = n_tr
    f["misc/it_range"] = np.array([it_lo, it_hi])
    f["misc/propagation_direction"] = "z"
    f.close()


def tracksFromOPMD_old(ts, pt, ref_iteration, fname=None, species=None, dNp=None,
                       Np_select=None, maxRaduis=None, Nit_min=None, Nit_max=None,
                       verbose=True):
    """The earlier openPMD reader: weights of the ``Np_select`` first particles
    or of every ``dNp``-th one, iterations strictly between ``Nit_min`` and
    ``Nit_max``; tracks longer than 8 steps go to ``fname`` (with their
    particle ids).  As in the reference, the positions recorded are those of
    the first ``Np_select`` particles in both cases.  Without ``fname`` the
    tracks of at least 8 steps are returned as ``(tracks, c dt)`` in the
    ``[x, y, z, ux, uy, uz, w, it_start]`` format ``calculate_spectrum``
    takes (the reference's list-building there raises a TypeError)."""
    Np = pt.N_selected
    w_select, = ts.get_particle(var_list=["w"], select=pt, species=species,
                                iteration=ref_iteration)
    if Np_select is None and dNp is None:
        print("Either Np_select or dNp can be used. Choosing all particles.")
        Np_select = w_select.size
    if Np_select is not None and dNp is not None:
        print("Only one of Np_select and dNp can be used. Stopping here.")
        return None
    if Np_select is not None:
        w_select = w_select[:Np_select]
    if dNp is not None:
        w_select = w_select[::dNp]
        Np_select = w_select.size

    iterations = ts.iterations.copy()
    keep = np.ones(iterations.size, dtype=bool)
    if Nit_min is not None:
        keep &= iterations > Nit_min
    if Nit_max is not None:
        keep &= iterations < Nit_max
    iterations = iterations[keep]
    dt = (ts.t[1] - ts.t[0]) * c

    tracks = np.zeros((iterations.size, Np_select, 7), dtype=np.double)
    nsteps = np.zeros(Np_select, dtype=np.int64)
    it_start = np.zeros(Np_select, dtype=np.int64)
    for it, iteration in enumerate(iterations):
        x, y, z, ux, uy, uz, id = ts.get_particle(
            var_list=["x", "y", "z", "ux", "uy", "uz", "id"], select=pt,
            iteration=iteration, species=species)
        if x.size < Np:
            continue
        record_particles_first(tracks, nsteps, it, it_start, x, y, z, ux, uy, uz, id,
                               Np_select)
        if verbose:
            print(f"Done {it / len(iterations) * 100: 0.1f}%", end="\r", flush=True)
    if verbose:
        print(f"Done reading {Np_select} particles")

    if fname is not None:
        f = _h5().File(fname, mode="w")
        n_tr, it_hi = 0, 0
        for ip in range(Np_select):
            n = nsteps[ip]
            if n <= 8:
                continue
            g = f"tracks/{n_tr:d}/"
            for k, name in enumerate(list(_COORDS) + ["id"]):
                f[g + name] = tracks[:n, ip, k]
            f[g + "w"] = w_select[ip]
            f[g + "it_start"] = it_start[ip]
            it_hi = max(it_hi, it_start[ip] + n)
            n_tr += 1
        f["misc/cdt"] = dt
        f["misc/N_particles"] = n_tr
        f["misc/it_range"] = np.array([it_start.min(), it_hi])
        f["misc/propagation_direction"] = "z"
        f.close()
        return None
    out = []
    for ip in range(Np_select):
        n = nsteps[ip]
        if n < 8:
            continue
        out.append([tracks[:n, ip, k].copy() for k in range(6)]
                   + [w_select[ip], int(it_start[ip])])
    return out, dt


def tracksFromVSIM(file_vsim, file_synchrad, cdt, length_unit=1, dNit=1, dNp=None,
                   Np_select=None, verbose=True):
    """A VSIM tracks file (dataset ``tracks`` [Nt, Np, 6] of z, y, x, uz, uy,
    ux in SI units) converted to a SynchRad track file: z-propagation axes,
    lengths divided by ``length_unit``, momenta by c, every ``dNit``-th
    iteration, every ``dNp``-th particle (then the first ``Np_select``); a
    particle's steps are those with x > 0, tracks longer than 8 steps are
    written with weight 1."""
    h5 = _h5()
    dt = cdt / length_unit
    src = h5.File(file_vsim, mode="r")
    dst = h5.File(file_synchrad, mode="w")
    n_p = src["tracks"].shape[1]
    particles = np.arange(n_p)
    if dNp is not None:
        particles = particles[::dNp]
    if Np_select is not None:
        particles = particles[:Np_select]
    n_tr, it_lo, it_hi = 0, np.inf, 0
    for ip in particles:
        z, y, x, uz, uy, ux = np.asarray(src["tracks"][::dNit, ip, :]).T
        inside = np.flatnonzero(x > 0)
        first = inside[0]
        it_lo = min(it_lo, first)
        if inside.size > 8:
            g = f"tracks/{n_tr:d}/"
            for name, v, scale in (("x", x, length_unit), ("y", y, length_unit),
                                   ("z", z, length_unit), ("ux", ux, c), ("uy", uy, c),
                                   ("uz", uz, c)):
                dst[g + name] = v[inside] / scale
            dst[g + "w"] = 1.0
            dst[g + "it_start"] = first
            n_tr += 1
            it_hi = max(it_hi, first + inside.size)
    dst["misc/cdt"] = dt * dNit
    dst["misc/N_particles"] = n_tr
    dst["misc/it_range"] = np.array([it_lo, it_hi])
    dst["misc/propagation_direction"] = "z"
    src.close()
    dst.close()
    if verbose:
        print(f"written {n_tr} tracks to {file_synchrad}")
