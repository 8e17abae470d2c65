"""``SynchRad``: the reference's calculator API on the GB300 CUDA library.

Same constructor, ``Args`` keys, ``calculate_spectrum`` signature, result
arrays (``self.Data['radiation'][key]``, float64, shape
``(nSnaps, nOmega, nTheta|nR, nPhi)``), ``total_weight``, ``snap_iterations``
and HDF5 layout as ``synchrad/calc.py``.  ``Args['dtype']`` keeps the
reference's meanings ('double': the plain FP64 kernel, 'float': FP32, with
``Args['native']`` for the fast intrinsics) and adds 'mixed': FP32 bulk
arithmetic with double-float phase and compensated sums, FP64 results; and
'double-float': double-float arithmetic throughout (far field), FP64-class
results on the FP32 pipe.

Differences from the reference, all deliberate:
  * one batched GPU call per ``calculate_spectrum`` instead of one OpenCL
    launch per track; the per-track launch semantics (``it_range`` rules,
    snapshot state machine, weight scaling) are kept exactly;
  * distribution over processes uses ``torch.distributed`` (when initialised)
    in place of mpi4py: tracks are strided over ranks and the spectra are
    summed on rank 0, as ``synchrad/calc.py:212, 236, 560-571`` do;
  * tracks whose ``itEnd`` or step count is 0 are rejected with ValueError (the
    reference's unsigned loop bounds wrap around for them).
Addition: ``Args['autotune']`` (True, or a budget in ms) tunes the work shape
of the 'mixed' kernels once per batch size before its first evaluation.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .batch import (TrackStream, Workspace, autotune, make_grid, pack_tracks, plan_chunks,
                    precision_id, run_spectrum, snap_iterations)
from .utils import Utilities

VEC_COMPS = {
    "cartesian": ["x", "y", "z"],
    "cartesian_complex": ["xre", "xim", "yre", "yim", "zre", "zim"],
    "spheric": ["r", "theta", "phi"],
    "spheric_complex": ["rre", "rim", "thetare", "thetaim", "phire", "phiim"],
    "total": ["total"],
}


def _dist():
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist
    except Exception:  # pragma: no cover
        pass
    return None


class SynchRad(Utilities):
    """Synchrotron-radiation calculator (see ``synchrad/calc.py:21-100``)."""

    def __init__(self, Args={}, file_spectrum=None):
        dist = _dist()
        if dist is not None:
            self.comm = dist
            self.rank = dist.get_rank()
            self.size = dist.get_world_size()
        else:
            self.rank = 0
            self.size = 1
        if file_spectrum is None:
            self._init_args(Args)
            self._init_comm()
            self._init_data()
            self._compile_kernels()
        else:
            self._read_args(file_spectrum)

    # ------------------------------------------------------------------
    def calculate_spectrum(self, particleTracks=[], file_tracks=None, timeStep=None,
                           comp="total", L_screen=None, Np_max=None, it_range=None,
                           nSnaps=1, sigma_particle=0, weights_normalize=None,
                           file_spectrum=None, verbose=True):
        """Compute the spectrum of ``particleTracks`` (or of ``file_tracks``).

        Same arguments and effects as ``synchrad/calc.py:101-290``.
        """
        if comp not in VEC_COMPS:
            raise ValueError(f"unknown comp {comp!r}")
        if self.Args["mode"] == "near" and comp.startswith("spheric"):
            raise ValueError("spheric components are far-field only")
        self.Args["sigma_particle"] = self.dtype(sigma_particle)
        if self.Args["mode"] == "near":
            if L_screen is not None:
                self.Args["L_screen"] = L_screen
            else:
                print("Define L_screen argument for near-field calculation")

        nSnaps = np.uint32(nSnaps)
        self._init_raditaion(comp, nSnaps)

        if timeStep is not None:
            self.Args["timeStep"] = self.dtype(timeStep)
        if it_range is not None:
            it_range = tuple(it_range)

        if file_tracks is not None:
            particleTracks, it_range = self._read_tracks(file_tracks, it_range, nSnaps,
                                                         Np_max, verbose)
        else:
            if it_range is not None:
                self.snap_iterations = snap_iterations(it_range, nSnaps)
            elif self.rank == 0 and verbose:
                print("Separate it_range for each track will be used")
            Np = len(particleTracks)
            if Np_max is not None:
                Np = min(Np_max, Np)
            particleTracks = particleTracks[:Np][self.rank::self.size]

        self.total_weight = 0.0
        if weights_normalize in ("mean", "max"):
            weights = [track[6] for track in particleTracks]
            weight_norm = np.mean(weights) if weights_normalize == "mean" else np.max(weights)
        for track in particleTracks:
            if weights_normalize in ("mean", "max"):
                track[6] /= weight_norm
            elif weights_normalize == "ones":
                track[6] = 1.0
            self.total_weight += track[6]

        if particleTracks:
            self._run_tracks(particleTracks, comp, nSnaps, it_range)
        elif it_range is None:
            self.snap_iterations = np.zeros(0, dtype=np.uint32)

        self._spectr_from_device(nSnaps)
        if self.size > 1:
            self._gather_result_dist()

        if file_spectrum is not None and self.rank == 0:
            self._write_hdf5(file_spectrum)

    # ------------------------------------------------------------------
    def _run_tracks(self, tracks, comp, nSnaps, it_range):
        dt = self.Args.get("timeStep")
        if dt is None:
            raise ValueError("timeStep is not defined")
        name = self.Args["dtype"]
        if name == "float":
            np_dtype = np.float32
        elif name == "double":
            np_dtype = np.float64
        else:  # mixed, double-float: FP32 tracks stay FP32, others FP64
            all32 = all(np.asarray(t[k]).dtype == np.float32 for t in tracks for k in range(6))
            np_dtype = np.float32 if all32 else np.float64
        if it_range is None:
            last = int(np.asarray(tracks[-1][0]).size)
            self.snap_iterations = snap_iterations((0, last), nSnaps)
        outs = [self._spect_dev[k] for k in VEC_COMPS[comp]]
        prec = precision_id(name, "native" in self.Args)
        tune = self.Args.get("autotune")  # not a reference key: True or a budget in ms
        done = self.__dict__.setdefault("_tuned", set())
        if self.device.type != "cuda":  # host-placed arrays (checks of the host logic)
            batch = pack_tracks(tracks, np_dtype, int(nSnaps), float(dt), it_range=it_range,
                                device=self.device)
            self._h2d_bytes = batch.h2d_bytes
            run_spectrum(batch, self._grid_dev, comp, prec, outs, workspace=self._workspace)
            return
        cur = torch.cuda.current_stream(self.device)
        if getattr(self, "_stream", None) is None:
            self._stream = TrackStream(self.device)
            self._lanes = ((torch.cuda.Stream(self.device), self._workspace),
                           (torch.cuda.Stream(self.device), Workspace(self.device)))
        plan = plan_chunks([np.asarray(t[0]).size for t in tracks], np.dtype(np_dtype).itemsize)
        # One chunk: everything on the current stream.  Several: chunks
        # alternate between two compute streams, each with its own workspace
        # and accumulator (the second one added in at the end), so that a
        # chunk's launch fills the SMs its predecessor's tail frees; the host
        # packs and copies the next chunk meanwhile.
        if len(plan) == 1:
            lanes = [(cur, self._workspace, outs)]
        else:
            extra = [torch.zeros_like(o) for o in outs]
            lanes = [(self._lanes[0][0], self._lanes[0][1], outs),
                     (self._lanes[1][0], self._lanes[1][1], extra)]
            for s_, _, o_ in lanes:
                s_.wait_stream(cur)  # outputs zeroed on the current stream
                for t_ in o_:
                    t_.record_stream(s_)
        # each call's kernel status word is or-ed into a flag per lane, read
        # once at the end (a read per chunk would serialise the streams)
        sticky = torch.zeros(len(lanes), dtype=torch.int32, device=self.device)
        self._h2d_bytes = 0
        chunks = self._stream.chunks(tracks, np_dtype, int(nSnaps), float(dt), it_range=it_range,
                                     plan=plan, compute_streams=[ln[0] for ln in lanes])
        for i, (batch, _, stream) in enumerate(chunks):
            _, wsp, o_ = lanes[i % len(lanes)]
            self._h2d_bytes += batch.h2d_bytes
            with torch.cuda.stream(stream):
                if tune and name == "mixed":
                    key = (batch.n_tracks, batch.total_steps, comp, int(nSnaps))
                    if key not in done:
                        budget = 3000.0 if tune is True else float(tune)
                        autotune(batch, self._grid_dev, comp, prec, budget, stream=stream)
                        done.add(key)
                run_spectrum(batch, self._grid_dev, comp, prec, o_, workspace=wsp, stream=stream)
                if wsp.buf is not None:
                    # the buffer may have been allocated on another stream: its
                    # memory is not handed out again before this stream's work
                    wsp.buf.record_stream(stream)
                    if prec == _lib.SR_PREC_MIXED:
                        sticky[i % len(lanes)].bitwise_or_(wsp.buf[:4].view(torch.int32)[0])
        if len(lanes) > 1:
            for s_, _, _ in lanes:
                cur.wait_stream(s_)
            for o, e in zip(outs, lanes[1][2]):
                o += e
        if int(sticky.max().item()) != 0:
            raise _lib.SynchRadError(_lib.SR_ERR_TIMEOUT,
                                     "a kernel wait on a staged copy ran out of time; the "
                                     "spectrum is incomplete")

    def _read_tracks(self, file_tracks, it_range, nSnaps, Np_max, verbose):
        """synchrad/calc.py:186-219 (needs h5py)."""
        import h5py

        with h5py.File(file_tracks, "r") as f:
            self.Args["timeStep"] = self.dtype(f["misc/cdt"][()])
            if it_range is None:
                if "it_range" in f["misc"].keys():
                    it_range = tuple(f["misc/it_range"][()])
                    self.snap_iterations = snap_iterations(it_range, nSnaps)
                    if self.rank == 0 and verbose:
                        print("it_range from the input file will be used")
                elif self.rank == 0 and verbose:
                    print("Separate it_range for each track will be used")
            else:
                self.snap_iterations = snap_iterations(it_range, nSnaps)
            Np = f["misc/N_particles"][()]
            if Np_max is not None:
                Np = min(Np_max, Np)
            cmps = ("x", "y", "z", "ux", "uy", "uz", "w", "it_start")
            tracks = []
            for ip in np.arange(Np)[self.rank::self.size]:
                tracks.append([f[f"tracks/{ip:d}/{c}"][()] for c in cmps])
        if self.rank == 0 and verbose:
            print("Tracks are loaded")
        return tracks, it_range

    def _write_hdf5(self, file_spectrum):
        """synchrad/calc.py:274-290 (needs h5py)."""
        import h5py

        with h5py.File(file_spectrum, "w") as f_out:
            for key in self.Data["radiation"].keys():
                f_out["radiation/" + key] = self.Data["radiation"][key]
            for key in self.Args.keys():
                if key in ("grid", "ctx"):
                    continue
                f_out["Args/" + key] = self.Args[key]
            f_out["snap_iterations"] = np.asarray(self.snap_iterations)
            f_out["total_weight"] = self.total_weight
        print(f"Spectrum is saved to {file_spectrum}")

    # ------------------------------------------------------------------
    def _init_args(self, Args):
        """Grid construction, synchrad/calc.py:355-451."""
        self.Args = Args
        if "mode" not in self.Args.keys():
            self.Args["mode"] = "far"
        if "dtype" not in self.Args:
            self.Args["dtype"] = "double"
        if self.Args["dtype"] in ("double", "mixed", "double-float"):
            self.dtype = np.double
        elif self.Args["dtype"] == "float":
            self.dtype = np.single
        else:
            raise ValueError(f"unknown dtype {self.Args['dtype']!r}")
        if self.Args["mode"] not in ("far", "near"):
            raise ValueError(f"unknown mode {self.Args['mode']!r}")
        if self.Args["dtype"] == "double-float" and self.Args["mode"] != "far":
            raise ValueError("dtype 'double-float' evaluates the far field only")
        if self.Args["dtype"] == "float":
            if self.Args["mode"] == "far":
                print("WARNING: Chosen single precision should be "
                      "used with care for the farfield calculations\n")
            else:
                print("WARNING: Chosen single precision is not "
                      "recommended for the nearfield calculations\n")
        if "ctx" not in self.Args.keys():
            self.Args["ctx"] = None

        self.Args["gridNodeNums"] = self.Args["grid"][-1]
        self.Args["numGridNodes"] = int(np.prod(self.Args["gridNodeNums"]))
        No = self.Args["gridNodeNums"][0]
        omega_min, omega_max = self.Args["grid"][0]
        if "Features" not in self.Args.keys():
            self.Args["Features"] = []
        omega = np.r_[omega_min:omega_max:No * 1j]
        for feature in self.Args["Features"]:
            if feature == "wavelengthGrid":
                self.Args["wavelengths"] = np.r_[1.0 / omega_max:1.0 / omega_min:No * 1j]
                omega = 1.0 / self.Args["wavelengths"]
                break
            elif feature == "logGrid":
                d_log_w = np.log(omega_max / omega_min) / (No - 1.0)
                omega = omega_min * np.exp(d_log_w * np.arange(No))
                break
        self.Args["omega"] = omega.astype(self.dtype)
        if No > 1:
            self.Args["dw"] = np.abs(omega[1:] - omega[:-1])
        else:
            self.Args["dw"] = np.array([1.0], dtype=self.dtype)

        if self.Args["mode"] == "far":
            Nt, Np = self.Args["gridNodeNums"][1:]
            theta_min, theta_max = self.Args["grid"][1]
            phi_min, phi_max = self.Args["grid"][2]
            theta = np.r_[theta_min:theta_max:Nt * 1j]
            phi = phi_min + (phi_max - phi_min) / Np * np.arange(Np)
            self.Args["dth"] = theta[1] - theta[0] if Nt > 1 else self.dtype(1.0)
            self.Args["dph"] = phi[1] - phi[0] if Np > 1 else self.dtype(1.0)
            self.Args["theta"] = theta.astype(self.dtype)
            self.Args["phi"] = phi.astype(self.dtype)
            self.Args["dV"] = self.Args["dw"] * self.Args["dth"] * self.Args["dph"]
        else:
            Nr, Np = self.Args["gridNodeNums"][1:]
            r_min, r_max = self.Args["grid"][1]
            phi_min, phi_max = self.Args["grid"][2]
            radius = np.r_[r_min:r_max:Nr * 1j]
            phi = phi_min + (phi_max - phi_min) / Np * np.arange(Np)
            self.Args["dr"] = radius[1] - radius[0] if Nr > 1 else 1.0
            self.Args["dph"] = phi[1] - phi[0] if Np > 1 else 1.0
            self.Args["phi"] = phi.astype(self.dtype)
            self.Args["radius"] = radius.astype(self.dtype)
            self.Args["dV"] = self.Args["dw"] * self.Args["dr"] * self.Args["dph"]

    def _init_comm(self):
        """Device selection (the CUDA counterpart of synchrad/calc.py:513-558).

        ``ctx``: None -> the current CUDA device; 'mpi' -> device = local rank;
        [platform, device] -> that device index; False -> no device.
        """
        ctx = self.Args["ctx"]
        self.device = None
        if ctx is False:
            self.dev_type, self.dev_name, self.plat_name = "Starting without", "", "None"
        else:
            if not torch.cuda.is_available():
                raise RuntimeError("synchrad_gb300 needs a CUDA device (none is visible)")
            if ctx is None:
                idx = torch.cuda.current_device()
            elif ctx == "mpi":
                idx = self.rank % torch.cuda.device_count()
            else:
                idx = int(ctx[-1])
            self.device = torch.device("cuda", idx)
            self.dev_type = "GPU"
            self.dev_name = torch.cuda.get_device_name(idx)
            self.plat_name = "CUDA"
        if self.rank == 0:
            print(f"Running on {self.size} devices")
            print(f"  {self.dev_type} device: {self.dev_name}")
            print(f"Platform: {self.plat_name}\nCompiler: synchrad_gb300 sm_103a")

    def _init_data(self):
        """Device axes, synchrad/calc.py:486-512."""
        self.Data = {}
        self._workspace = Workspace(self.device) if self.device is not None else None
        if self.device is None:
            return
        om = self.dtype(2 * np.pi) * self.Args["omega"]
        if self.Args["mode"] == "far":
            axes = (om, np.sin(self.Args["theta"]), np.cos(self.Args["theta"]),
                    np.sin(self.Args["phi"]), np.cos(self.Args["phi"]))
        else:
            axes = (om, self.Args["radius"], np.sin(self.Args["phi"]), np.cos(self.Args["phi"]))
        self._host_axes = [np.ascontiguousarray(a) for a in axes]

    def _compile_kernels(self):
        """Loads the CUDA library (the OpenCL JIT of synchrad/calc.py:605-624)."""
        if self.device is None:
            return
        _lib.lib()

    def _init_raditaion(self, comp, nSnaps):
        """Result arrays and FormFactor, synchrad/calc.py:453-484."""
        shape = (int(nSnaps),) + tuple(self.Args["gridNodeNums"][::-1])
        self.Args["comp"] = comp
        if self.Args["mode"] == "near":
            self.Args["theta"] = np.arctan2(self.Args["radius"], self.Args["L_screen"])
        self.Data["radiation"] = {}
        exp_factor = self.dtype(-0.5) * (self.dtype(2 * np.pi) * self.Args["omega"]
                                         * self.Args["sigma_particle"]) ** 2
        form_factor = np.exp(exp_factor)
        self.Data["FormFactor"] = form_factor
        if self.device is None:
            raise RuntimeError("SynchRad was created without a device (ctx=False)")
        tdt = torch.float32 if self.Args["dtype"] == "float" else torch.float64
        self._spect_dev = {k: torch.zeros(shape, dtype=tdt, device=self.device)
                           for k in VEC_COMPS[comp]}
        self.Data["radiation"] = self._spect_dev
        n = tuple(int(v) for v in self.Args["gridNodeNums"])
        L = self.Args.get("L_screen", 0.0) if self.Args["mode"] == "near" else 0.0
        self._grid_dev = make_grid(self.Args["mode"], self._host_axes, n, tdt, self.device,
                                   form_factor=np.ascontiguousarray(form_factor),
                                   L_screen=self.dtype(L) if L is not None else 0.0)

    def _spectr_from_device(self, nSnaps):
        """synchrad/calc.py:573-577: to host, (nSnaps, nOmega, nTheta, nPhi)
        float64; the axis swap and the widening of FP32 spectra are done on
        the device (both exact), before the copy."""
        out = {}
        for key, t in self._spect_dev.items():
            host = t.transpose(-1, -3).to(torch.float64).contiguous().cpu()
            out[key] = host.numpy()
        self.Data["radiation"] = out

    def _gather_result_dist(self):
        """Sum the ranks' spectra and weights on rank 0 (synchrad/calc.py:560-571).

        As there, only rank 0 holds the sums afterwards; the other ranks are
        left with zero spectra and ``total_weight`` None (the receive buffers
        of the reference's Reduce and the non-root result of its reduce)."""
        dist = self.comm
        # NCCL reduces device tensors only; gloo (and others) take host tensors
        on_dev = (str(dist.get_backend()).lower() == "nccl" and self.device is not None)
        for key in list(self.Data["radiation"].keys()):
            t = torch.from_numpy(self.Data["radiation"][key])
            if on_dev:
                t = t.to(self.device)
            dist.reduce(t, dst=0)
            summed = t.cpu().numpy()
            self.Data["radiation"][key] = summed if self.rank == 0 else np.zeros_like(summed)
        tw = torch.tensor([float(self.total_weight)], dtype=torch.float64,
                          device=self.device if on_dev else "cpu")
        dist.reduce(tw, dst=0)
        self.total_weight = float(tw[0]) if self.rank == 0 else None

    def _read_args(self, file_spectrum):
        """synchrad/calc.py:648-666 (needs h5py)."""
        import h5py

        if self.rank == 0:
            self.Data = {"radiation": {}}
            self.Args = {}
            with h5py.File(file_spectrum, "r") as f:
                for key in f["radiation"].keys():
                    self.Data["radiation"][key] = f["radiation/" + key][()]
                for key in f["Args"].keys():
                    self.Args[key] = f["Args/" + key][()]
                    if isinstance(self.Args[key], bytes):
                        self.Args[key] = self.Args[key].decode()
                self.snap_iterations = f["snap_iterations"][()]
                self.total_weight = f["total_weight"][()]
