"""Multi-rank path of SynchRad on CPU: two gloo ranks.

The reference strides tracks over MPI ranks and sums the spectra and the
total weight on rank 0 (synchrad/calc.py:212, 236, 560-571); SynchRad does
the same over torch.distributed.  Here each rank's per-track evaluation is
the oracle (the GPU kernels need a device), everything else is SynchRad's
own code: track striding, weight accumulation, the device-to-host layout
swap and the reduction on rank 0.  The result must equal the oracle's
single-process spectrum of all tracks; the other rank is left with zero
spectra and ``total_weight`` None, as after the reference's MPI reduction.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")

GRID = [(20.0, 60.0), (0.0, 0.08), (0.0, 2 * np.pi), (16, 5, 4)]


def _tracks():
    from synchrad_gb300 import workloads as wl
    rng = np.random.default_rng(4)
    out = []
    for i in range(5):
        tr = wl.undulator_track(12.0 + i, 0.4, 2 + i % 3, 1.0 / 16, x0=rng.normal(0, 0.02),
                                weight=float(rng.uniform(0.5, 1.5)))
        out.append(tr)
    return out


def _cpu_synchrad_class():
    from oracle import host as ohost
    from synchrad_gb300.calc import VEC_COMPS, SynchRad

    class CpuSynchRad(SynchRad):
        """SynchRad whose per-rank track evaluation runs the oracle on the CPU."""

        def _init_raditaion(self, comp, nSnaps):
            shape = (int(nSnaps),) + tuple(self.Args["gridNodeNums"][::-1])
            self.Args["comp"] = comp
            self._spect_dev = {k: torch.zeros(shape, dtype=torch.float64)
                               for k in VEC_COMPS[comp]}
            self.Data["radiation"] = self._spect_dev

        def _run_tracks(self, tracks, comp, nSnaps, it_range):
            args = {"grid": self.Args["grid"], "dtype": "double", "mode": self.Args["mode"]}
            rad, _, snaps, _ = ohost.calculate_spectrum(
                args, [list(t) for t in tracks], float(self.Args["timeStep"]), comp=comp,
                nSnaps=int(nSnaps), it_range=it_range, kind="port", nthreads=2)
            self.snap_iterations = snaps
            for k in self._spect_dev:  # host (nSnaps, nO, nT, nP) -> device order
                self._spect_dev[k] += torch.from_numpy(
                    np.ascontiguousarray(rad[k].swapaxes(-1, -3)))

    return CpuSynchRad


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cls = _cpu_synchrad_class()
        calc = cls({"grid": GRID, "dtype": "double", "ctx": False})
        assert calc.rank == rank and calc.size == world
        calc.calculate_spectrum(_tracks(), timeStep=1.0 / 16, comp="total", verbose=False)
        if rank == 0:
            np.save(os.path.join(out_dir, "total.npy"), calc.Data["radiation"]["total"])
            np.save(os.path.join(out_dir, "weight.npy"), np.array([calc.total_weight]))
        else:  # as after the reference's Reduce: zero spectra, no total weight
            spec = calc.Data["radiation"]["total"]
            np.save(os.path.join(out_dir, f"rank{rank}.npy"),
                    np.array([float(np.abs(spec).max()), spec.size,
                              float(calc.total_weight is None)]))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_match_one_process(tmp_path):
    import torch.multiprocessing as mp
    from oracle import host as ohost
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = np.load(tmp_path / "total.npy")
    weight = float(np.load(tmp_path / "weight.npy")[0])
    tracks = _tracks()
    args = {"grid": GRID, "dtype": "double", "mode": "far"}
    rad, total_weight, _, _ = ohost.calculate_spectrum(args, [list(t) for t in tracks], 1.0 / 16,
                                                       comp="total", kind="port", nthreads=2)
    exp = rad["total"]
    assert got.shape == exp.shape
    assert np.linalg.norm(got - exp) / np.linalg.norm(exp) < 1e-13
    assert weight == pytest.approx(total_weight, rel=1e-14)
    peak, size, weight_none = np.load(tmp_path / "rank1.npy")
    assert peak == 0.0 and size == exp.size and weight_none == 1.0
