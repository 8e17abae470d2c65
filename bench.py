"""Benchmark of the SynchRad radiation integral on GB300.

Metric: Gpt*steps/s = spectral points x sum over tracks of (steps - 1), per
second, / 1e9, for the mixed-precision far-field path, with its relative L2
error against the plain FP64 kernel stated alongside.

Default workload (the configuration the metric is quoted on): 1024 electrons,
gamma ~ N(400, 1%), planar undulator K = 1, offsets N(0, 2 um-eq), angles
N(0, 0.05/gamma), 4000 steps each, weights U[0.5, 1.5]; grid 512 omega x 64
theta x 64 phi over the first three harmonics; comp 'total'.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One "step" is one pass of the whole batch (every track, every point) through
``sr_spectrum`` with the tracks already resident in HBM; L2 is flushed (a
256 MB write) before every timed step.  ``e2e`` repeats the measurement through
the public API ``SynchRad.calculate_spectrum`` from host (numpy) tracks, with
the packing, host-to-device copies, kernels and the device-to-host read of the
spectrum inside the timed region.

Under torchrun (N > 1) each rank evaluates its own copy of the workload on its
GPU (tracks are independent; weak scaling, no collective in the timed loop);
the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gpt·steps/s (spectral pts × track steps), mixed vs FP64 at ≤1e-5 rel err"
UNIT = "Gpt·steps/s"
FLOPS_PER_UNIT = 14      # far field, mixed: 2 FMUL + 6 FFMA per point-step
ADJ_FLOPS_PER_UNIT = 22  # far adjoint: 8 FFMA (E and F sums) + 1 FMUL + 2 FFMA (rotation)
NEAR_ADJ_FLOPS_PER_UNIT = 42  # near adjoint: 18 FFMA (R0, I1, R2 x 3) + rotation
CANONICAL_FLOPS = 18     # the 3-component formulation's count


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="far", choices=["far", "near", "ragged", "adjoint", "near-adjoint"],
                    help="far: the headline configuration (default); near: 2048 helical "
                         "tracks on a screen at 20 undulator lengths; ragged: 8192 FP32 "
                         "betatron tracks of 500-20000 steps; adjoint: forward and "
                         "backward of sum(g * S) for 256 tracks x 2000 steps on 128 x 32 x 32")
    ap.add_argument("--forward-precision", default="mixed", choices=["mixed", "double-float"],
                    help="adjoint workloads: arithmetic of the differentiable forward "
                         "(double-float: FP64-class spectrum, far field)")
    ap.add_argument("--tracks", type=int, default=None)
    ap.add_argument("--seed", type=int, default=0,
                    help="seed of the synthetic tracks (numpy default_rng)")
    ap.add_argument("--track-steps", type=int, default=None)
    ap.add_argument("--grid", type=int, nargs=3, default=None)
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the work-shape autotuner (default shape)")
    ap.add_argument("--tune-budget-ms", type=float, default=6000.0)
    ap.add_argument("--no-graph", action="store_true",
                    help="direct sr_spectrum calls instead of CUDA-graph replay")
    ap.add_argument("--shape", type=int, nargs=4, default=None,
                    metavar=("K", "L", "STAGE", "SUBSETS"),
                    help="pin the work shape (points per lane, lanes per direction, steps per "
                         "stage, track subsets; 0 subsets = default) instead of tuning")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clocks and throttle reasons."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: str):
        import tempfile
        self.gpu = gpu_index
        self.proc = None
        fd, name = tempfile.mkstemp(prefix="sr_clocks_", suffix=".csv")
        os.close(fd)
        self.path = Path(name)

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = np.array([float(r[1]) for r in rows])
        smax = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        power = [float(r[3]) for r in rows if r[3] not in ("[N/A]", "")]
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(power) if power else None}


def make_workload(args):
    from synchrad_gb300 import workloads as wl
    kw = {"seed": args.seed}
    if args.tracks is not None:
        kw["n_tracks"] = args.tracks
    if args.grid is not None:
        kw["grid"] = tuple(args.grid)
    if args.workload == "far":
        if args.track_steps is not None:
            kw["n_steps"] = args.track_steps
        return wl.c2_far_mixed(**kw)
    if args.workload == "near":
        if args.track_steps is not None:
            kw["n_steps"] = args.track_steps
        return wl.c5_near_helical(**kw)
    if args.workload == "adjoint":
        if args.track_steps is not None:
            kw["n_steps"] = args.track_steps
        return wl.c4_adjoint(**kw)
    if args.workload == "near-adjoint":
        if args.track_steps is not None:
            kw["n_steps"] = args.track_steps
        return wl.c5_near_helical(**kw)
    if args.track_steps is not None:
        kw["steps_range"] = (max(2, args.track_steps // 40), args.track_steps)
    return wl.c3_betatron_ragged(**kw)


def flops_per_unit(w):
    """Algorithmic FP32 flops per point-step (the roofline's numerator): far
    field 18 (rotation 2 FMUL + 2 FFMA, three complex components 6 FFMA),
    near field 30 (rotation 6, two vectors x 3 components x Re/Im 12 FFMA)."""
    return 30 if w.args.get("mode", "far") == "near" else CANONICAL_FLOPS


def executed_flops_per_unit(w):
    """Flops the mixed kernels execute per point-step: the far field carries
    A on theta-hat and phi-hat only (n.amp = 0), 2 FMUL + 6 FFMA = 14."""
    return 30 if w.args.get("mode", "far") == "near" else FLOPS_PER_UNIT


# DRAM bytes of one launch of the dominant kernel on the full default
# workloads, from single-pass ncu captures (dram__bytes_read.sum,
# dram__bytes_write.sum) of
#   bench.py --workload W --steps 1 --warmup 1 --no-e2e --no-cpu --no-fp64 --no-graph --shape K L S N
# with the shape the autotuner picks for that workload.  Most of it is the
# per-warp compensated sums (written back from L2 on eviction) and the
# per-subset FP64 partial spectra; neither is on the critical path of these
# FP32-bound kernels (2-14 GB/s against ~7 TB/s).
NCU_TRAFFIC = {
    # workload: (read bytes, write bytes, tracks, (K, L, stage, subsets), kernel)
    "far": (1.12e9, 5.01e9, 1024, (32, 16, 64, 10), "far_mixed_kernel<32,8>"),
    "near": (5.97e9, 142.33e9, 2048, (16, 16, 128, 10), "near_mixed_kernel<16,8>"),
}


def launch_traffic(workload, args, n_tracks, shape):
    """DRAM bytes of one launch from the full-size ncu capture, or None where
    the capture does not describe this run (other tracks, steps or grid)."""
    if (workload not in NCU_TRAFFIC or args.track_steps is not None or args.grid is not None
            or args.seed != 0):
        return None, None
    rd, wr, nt, sh, src = NCU_TRAFFIC[workload]
    if n_tracks != nt:
        return None, None
    run_sh = (shape["points_per_lane"], shape["lanes_per_direction"],
              shape["steps_per_stage"], shape["track_subsets"])
    note = "" if run_sh == sh else f"; this run's shape {run_sh} differs"
    return (rd + wr,
            f"ncu capture of one full launch of {src} ({nt} tracks, shape K/L/stage/subsets "
            f"{sh}): dram__bytes_read.sum {rd:.4g} + dram__bytes_write.sum {wr:.4g}{note}")


def product_calc(w):
    """The product's own ``SynchRad`` for this workload's grid ('mixed'): its
    ``Args`` (grid construction) and host device axes (``_init_data``) feed
    the device-timed arms, so that they evaluate exactly the axes a user's
    ``calculate_spectrum`` call would."""
    import contextlib
    import io
    from synchrad_gb300.calc import SynchRad
    with contextlib.redirect_stdout(io.StringIO()):  # its device banner
        return SynchRad(dict(w.args, dtype="mixed"))


def product_grid(w, device):
    import torch
    from synchrad_gb300.batch import make_grid
    calc = product_calc(w)
    n = tuple(int(v) for v in calc.Args["gridNodeNums"])
    grid = make_grid(calc.Args["mode"], calc._host_axes, n, torch.float64, device,
                     L_screen=w.L_screen or 0.0)
    return calc, grid, n


def mixed_vs_oracle(w, n_tracks=2, sub=(8, 8)):
    """Relative L2 and max relative error of the mixed path (``SynchRad``,
    dtype 'mixed') against the FP64 CPU oracle (the reference kernels'
    arithmetic in C) on a bounded sample: the first tracks, whole, on the
    full omega axis and the configuration's theta (or R) and phi ranges on
    ``sub`` nodes (the last theta / R node included)."""
    import contextlib
    import io
    from oracle import host
    from synchrad_gb300.calc import SynchRad
    g = w.args["grid"]
    grid = [g[0], g[1], g[2], (g[3][0],) + tuple(sub)]
    mode = w.args.get("mode", "far")
    tracks = [list(t) for t in w.tracks[:n_tracks]]
    t0 = time.perf_counter()
    ref, *_ = host.calculate_spectrum({"grid": grid, "dtype": "double", "mode": mode},
                                      [list(t) for t in tracks], w.time_step,
                                      L_screen=w.L_screen, kind="port")
    el = time.perf_counter() - t0
    with contextlib.redirect_stdout(io.StringIO()):
        calc = SynchRad({"grid": grid, "dtype": "mixed", "mode": mode})
        calc.calculate_spectrum([list(t) for t in tracks], timeStep=w.time_step,
                                L_screen=w.L_screen, verbose=False)
    got = calc.Data["radiation"]["total"].ravel()
    exp = ref["total"].ravel()
    rel = float(np.linalg.norm(got - exp) / np.linalg.norm(exp))
    big = np.abs(exp) > 1e-3 * np.abs(exp).max()
    maxrel = float(np.max(np.abs(got[big] - exp[big]) / np.abs(exp[big])))
    return {"against": "FP64 CPU oracle (the reference kernels' arithmetic, C)",
            "sample": (f"first {n_tracks} tracks (whole), full omega axis x {sub[0]} x "
                       f"{sub[1]} directions or screen points over the configuration's "
                       f"ranges (last theta / R node included); oracle {el:.1f} s"),
            "rel_l2": rel, "max_rel": maxrel,
            "max_rel_floor": "points above 1e-3 of the sample's maximum",
            "tolerance_rel_l2": 1e-5}


def cpu_sample(w, n_tracks=4, sub=(16, 16)):
    """A bounded sample of the workload for the CPU oracle: the first tracks on
    the full omega axis and a sub-grid of directions."""
    args = dict(w.args)
    nO, nT, nP = args["grid"][-1]
    (t0, t1), (p0, p1) = args["grid"][1], args["grid"][2]
    # the first sub[0] theta nodes and sub[1] phi nodes of the full grid
    dth = (t1 - t0) / (nT - 1) if nT > 1 else 0.0
    dph = (p1 - p0) / nP
    g = [args["grid"][0], (t0, t0 + dth * (sub[0] - 1)), (p0, p0 + dph * sub[1]),
         (nO, sub[0], sub[1])]
    tracks = [[np.asarray(a, np.float64) for a in t[:6]] + list(t[6:])
              for t in w.tracks[:n_tracks]]
    return {"grid": g, "dtype": "double", "mode": args.get("mode", "far")}, tracks


def time_cpu_oracle(w, nthreads, n_tracks=4, sub=(16, 16), kind=None):
    import oracle
    from oracle import host
    if kind is None:
        kind = "reference" if oracle.ref_available() else "port"
    lib_kind = "ref" if kind == "reference" else "port"
    a, tracks = cpu_sample(w, n_tracks, sub)
    t0 = time.perf_counter()
    host.calculate_spectrum(a, tracks, w.time_step, comp="total", kind=lib_kind,
                            nthreads=nthreads, L_screen=w.L_screen)
    el = time.perf_counter() - t0
    pts = int(np.prod(a["grid"][-1])) * sum(len(t[0]) - 1 for t in tracks)
    return pts / el / 1e9, el, pts, kind


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def single_core_baseline(w, kind=None):
    """The oracle on one thread over a smaller sample of the same workload."""
    v1, el1, _, kind = time_cpu_oracle(w, 1, n_tracks=1, sub=(8, 8), kind=kind)
    return {"value": v1, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": (f"first track on the full omega axis x 8 x 8 directions or screen "
                       f"points, FP64, 1 thread, {el1:.1f} s")}


def reference_arm(args):
    """--impl reference: the reference's CPU implementation of the path."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    w = make_workload(args)
    nth = os.cpu_count() or 1
    vals = []
    kind = None
    for i in range(args.warmup + args.steps):
        v, el, pts, kind = time_cpu_oracle(w, nth, n_tracks=2, sub=(8, 16))
        if i >= args.warmup:
            vals.append((v, el))
    v = float(np.median([x[0] for x in vals]))
    ms = float(np.mean([x[1] for x in vals])) * 1e3
    sample = (f"first 2 tracks on the full omega axis x 8 x 16 directions or screen "
              f"points (the first nodes of the grid), FP64, {nth} threads")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": w.name, "sample": sample},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth,
                             "kind": "reference" if kind == "reference" else "port",
                             "sample": sample, "model": cpu_model(),
                             "single_core": single_core_baseline(w, kind)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def adjoint_main(args):
    """Forward (mixed far field, amplitudes kept), loss and backward (adjoint
    kernel) on the adjoint workload.  The loss is the weighted L2 misfit
    L = sum(((S - T) / max T)^2) against a target spectrum T of the same tracks
    with seeded perturbations (x, y and momenta 1e-3 relative), computed once
    before timing.  One step = forward + loss + backward, L2 flushed before
    each.  Reports the forward and backward times and their ratio.

    ``--workload near-adjoint``: the near-field workload (screen at 20
    undulator lengths) with the on-screen energy integral of
    Utilities.get_energy as the loss (its quadrature weights as dL/dS)."""
    import torch
    from synchrad_gb300 import _lib
    from synchrad_gb300.autograd import make_layout, total_spectrum_fn

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    device = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(device)
    L = _lib.lib()
    w = make_workload(args)
    calc = product_calc(w)
    nO, nT, nP = (int(v) for v in calc.Args["gridNodeNums"])
    mode = w.args.get("mode", "far")
    lengths = [len(t[0]) for t in w.tracks]
    layout = make_layout(lengths, w.time_step, calc._host_axes, (nO, nT, nP), device,
                         mode=mode, L_screen=w.L_screen or 0.0,
                         precision=args.forward_precision)
    spectrum = total_spectrum_fn(mode)
    coords = [torch.tensor(np.concatenate([np.asarray(t[c], np.float64) for t in w.tracks]),
                           device=device, requires_grad=True) for c in range(6)]
    wt = torch.tensor([float(t[6]) for t in w.tracks], dtype=torch.float64, device=device,
                      requires_grad=True)
    if mode == "far":
        from synchrad_gb300 import workloads as wl
        tgt = wl.perturbed_tracks(w.tracks, 1e-3, seed=1)
        tgt_coords = [torch.tensor(np.concatenate([np.asarray(t[c], np.float64) for t in tgt]),
                                   device=device) for c in range(6)]
        with torch.no_grad():
            target = spectrum(*tgt_coords, wt.detach(), layout)
        inv_scale = 1.0 / float(target.max())

        def loss_of(S):
            return (((S - target) * inv_scale) ** 2).sum()
        loss_name = ("sum(((S - T) / max T)^2), T from the tracks with x, y and momenta "
                     "perturbed 1e-3 relative (seed 1)")
    else:
        calc.Args["comp"] = "total"
        q = torch.tensor(np.ascontiguousarray(calc.get_energy_weights(lambda0_um=1.0)
                                              .transpose(2, 1, 0)), device=device)

        def loss_of(S):
            return (q * S).sum()
        loss_name = "on-screen radiated energy (Utilities.get_energy quadrature, lambda0 1 um)"
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)
    pt_steps = w.pt_steps
    tune = None
    if not args.no_tune and args.forward_precision == "mixed":  # the forward's work shape
        from synchrad_gb300.autograd import _tracks_struct
        from synchrad_gb300.batch import autotune
        t0 = time.perf_counter()
        tune = autotune(_tracks_struct([c.detach() for c in coords], wt.detach(), layout),
                        layout.grid, "total", _lib.SR_PREC_MIXED, args.tune_budget_ms, stream)
        tune["wall_s"] = time.perf_counter() - t0

    def one_step(ev=None):
        flush.fill_(1.0)
        for c in coords + [wt]:
            c.grad = None
        if ev:
            ev[0].record(stream)
        S = spectrum(*coords, wt, layout)
        if ev:
            ev[1].record(stream)
            _lib.check(L.sr_timing_enable(1))
        loss = loss_of(S)
        loss.backward()
        if ev:
            _lib.check(L.sr_timing_enable(0))
            ev[2].record(stream)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    _lib.check(L.sr_timing_read(None, None))
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(device).uuid)
    except Exception:
        gpu_id = str(device.index)
    with ClockSampler(gpu_id) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e_start = torch.cuda.Event(enable_timing=True)
        e_end = torch.cuda.Event(enable_timing=True)
        e_start.record(stream)
        for k in range(args.steps):
            one_step(evs[k])
        e_end.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    kern_ms = ctypes.c_double(0)
    kern_n = ctypes.c_int(0)
    _lib.check(L.sr_timing_read(ctypes.byref(kern_ms), ctypes.byref(kern_n)))
    elapsed = e_start.elapsed_time(e_end)
    if dist:
        t = torch.tensor([elapsed], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    fwd_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in evs]))
    bwd_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in evs]))
    ms_per_step = elapsed / args.steps
    tf_s = ctypes.c_double(0)
    tf_p = ctypes.c_double(0)
    _lib.check(L.sr_probe_fp32_peak(ctypes.byref(tf_s), ctypes.byref(tf_p),
                                    ctypes.c_void_p(stream.cuda_stream)))
    peak = max(tf_s.value, tf_p.value)
    kern_avg = kern_ms.value / max(kern_n.value, 1)
    fpu = ADJ_FLOPS_PER_UNIT if mode == "far" else NEAR_ADJ_FLOPS_PER_UNIT
    kname = "adj_far_kernel" if mode == "far" else "nadj_kernel"
    achieved = pt_steps * fpu / (kern_avg * 1e-3) / 1e12
    if rank == 0:
        line = {"metric": ("Gpt·steps/s through forward + backward of a spectrum misfit loss "
                           "(far field)" if mode == "far" else
                           "Gpt·steps/s through forward + backward of the on-screen energy "
                           "(near field)"),
                "value": pt_steps * ws * args.steps / (elapsed * 1e-3) / 1e9, "unit": UNIT,
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None,
                "dtype": ("f32 (mixed: double-float phase, FP32 sums, FP64 gradients)"
                          if args.forward_precision == "mixed" else
                          "double-float forward (~48-bit, FP32 pipe); mixed adjoint, FP64 "
                          "gradients"),
                "data": "synthetic",
                "config": {"workload": w.name, "n_tracks": len(w.tracks), "seed": args.seed,
                           "steps_per_track": int(lengths[0]), "grid": [nO, nT, nP],
                           "pt_steps_per_step": pt_steps,
                           "loss": loss_name,
                           "forward_precision": args.forward_precision,
                           "l2": "flushed before every timed step (256 MB write, counted)",
                           "parallelism": f"replicas x{ws} (tracks independent)"},
                "adjoint": {"forward_ms": fwd_ms, "backward_ms": bwd_ms,
                            "backward_over_forward": bwd_ms / fwd_ms,
                            "adjoint_kernel_ms": kern_avg, "forward_autotune": tune},
                "e2e": None, "gpu_launches": 10 * args.steps,
                "clocks": clocks.summary(),
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak,
                             "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                             "traffic": None, "kernel": kname,
                             "flops_per_unit": fpu,
                             "peak_source": "measured on this GPU by sr_probe_fp32_peak"},
                "cpu_baseline": None}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.workload in ("adjoint", "near-adjoint"):
        adjoint_main(args)
        return
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    device = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(device)

    from synchrad_gb300 import _lib
    from synchrad_gb300.batch import (SpectrumGraph, Workspace, autotune, current_config,
                                      pack_tracks, run_spectrum)
    from synchrad_gb300.calc import SynchRad

    L = _lib.lib()
    w = make_workload(args)
    mode = w.args.get("mode", "far")
    _, grid, (nO, nT, nP) = product_grid(w, device)
    P = nO * nT * nP
    track_np = np.float32 if args.workload == "ragged" else np.float64
    batch = pack_tracks(w.tracks, track_np, 1, w.time_step, device=device)
    out = torch.zeros((1, nP, nT, nO), dtype=torch.float64, device=device)
    wsp = Workspace(device)
    pt_steps = w.pt_steps
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    tune = None
    if args.shape is not None:
        from synchrad_gb300.batch import set_config
        k_, l_, st_, ns_ = args.shape
        set_config(batch, grid, "total", _lib.SR_PREC_MIXED, k_, l_, st_, ns_)
    elif not args.no_tune:
        t0 = time.perf_counter()
        tune = autotune(batch, grid, "total", _lib.SR_PREC_MIXED, args.tune_budget_ms, stream)
        tune["wall_s"] = time.perf_counter() - t0
    shape = current_config(batch, grid, "total", _lib.SR_PREC_MIXED)
    graph = None
    if not args.no_graph:
        graph = SpectrumGraph(batch, grid, "total", _lib.SR_PREC_MIXED, [out], wsp)

    def one_step(direct=False):
        flush.fill_(1.0)
        out.zero_()
        if graph is not None and not direct:
            graph.launch(stream)
        else:
            run_spectrum(batch, grid, "total", _lib.SR_PREC_MIXED, [out], workspace=wsp,
                         stream=stream)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    _lib.check(L.sr_timing_read(None, None))  # clear
    if graph is None:
        _lib.check(L.sr_timing_enable(1))
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(device).uuid)
    except Exception:
        gpu_id = str(device.index)
    with ClockSampler(gpu_id) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            one_step()
        ev1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    _lib.check(L.sr_workspace_status(ctypes.c_void_p(wsp.buf.data_ptr()),
                                     ctypes.c_void_p(stream.cuda_stream)))
    elapsed_ms = ev0.elapsed_time(ev1)
    graph_spec = out.clone()
    if graph is not None:
        # the graph's kernels are not timed one by one: time the dominant kernel
        # on one direct call of the same shape
        _lib.check(L.sr_timing_enable(1))
        one_step(direct=True)
        torch.cuda.synchronize()
        assert torch.equal(out, graph_spec), "graph replay and direct call differ"
    _lib.check(L.sr_timing_enable(0))
    kern_ms = ctypes.c_double(0)
    kern_n = ctypes.c_int(0)
    _lib.check(L.sr_timing_read(ctypes.byref(kern_ms), ctypes.byref(kern_n)))
    if dist:
        t = torch.tensor([elapsed_ms], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    ms_per_step = elapsed_ms / args.steps
    value = pt_steps * ws * args.steps / (elapsed_ms * 1e-3) / 1e9
    mixed_spec = out.clone()

    # --- roofline of the dominant kernel (far_mixed_kernel) ---
    tf_s = ctypes.c_double(0)
    tf_p = ctypes.c_double(0)
    _lib.check(L.sr_probe_fp32_peak(ctypes.byref(tf_s), ctypes.byref(tf_p),
                                    ctypes.c_void_p(stream.cuda_stream)))
    kern_avg_ms = kern_ms.value / max(kern_n.value, 1)
    fpu = flops_per_unit(w)
    fpu_exec = executed_flops_per_unit(w)
    achieved = pt_steps * fpu / (kern_avg_ms * 1e-3) / 1e12
    achieved_exec = pt_steps * fpu_exec / (kern_avg_ms * 1e-3) / 1e12
    peak = max(tf_s.value, tf_p.value)
    clk = clocks.summary()
    kname = "near_mixed_kernel" if mode == "near" else "far_mixed_kernel"
    traffic, traffic_src = launch_traffic(args.workload, args, len(w.tracks), shape)
    roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak if peak else None,
                "traffic": traffic, "traffic_unit": "bytes per launch",
                "traffic_source": traffic_src,
                "kernel": (f"{kname} ({shape['points_per_lane']} omega points per lane, "
                           f"{shape['lanes_per_direction']} lanes per direction, 8 warps per CTA)"),
                "kernel_ms_avg": kern_avg_ms,
                "flops_per_unit": fpu,
                "flops_per_unit_source": ("algorithmic work per point-step of the "
                                          "three-component formulation (rotation 2 FMUL + "
                                          "2 FFMA, accumulation 6 FFMA)"
                                          if mode == "far" else
                                          "algorithmic work per point-step (rotation 6, "
                                          "two vectors x 3 components x Re/Im 12 FFMA)"),
                "flops_per_unit_executed": fpu_exec,
                "frac_executed": achieved_exec / peak if peak else None,
                "peak_source": ("measured on this GPU by sr_probe_fp32_peak (FFMA / FFMA2 "
                                f"throughput: {tf_s.value:.1f} / {tf_p.value:.1f} TFLOP/s); "
                                "MEASURED_PEAKS.json has no FP32 figure"),
                "peak_nominal_at_max_clock": (2 * 128 * torch.cuda.get_device_properties(device)
                                              .multi_processor_count
                                              * (clk.get("sm_max_mhz") or 2070) * 1e6 / 1e12)}

    # --- throughput of the plain FP64 CUDA kernel on a track subset, and the
    # mixed path's error against the FP64 CPU oracle on a bounded sample ---
    fp64 = None
    accuracy = None
    if not args.no_fp64:
        sub_tr = [[np.asarray(v, np.float64) for v in t[:6]] + list(t[6:]) for t in w.tracks[:2]]
        sb = pack_tracks(sub_tr, np.float64, 1, w.time_step, device=device)
        o64 = torch.zeros_like(out)
        omx = torch.zeros_like(out)
        run_spectrum(sb, grid, "total", _lib.SR_PREC_MIXED, [omx], workspace=wsp)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run_spectrum(sb, grid, "total", _lib.SR_PREC_DOUBLE, [o64], workspace=wsp)
        e1.record(stream)
        torch.cuda.synchronize()
        t64 = e0.elapsed_time(e1)
        pts64 = P * sum(len(t[0]) - 1 for t in sub_tr)
        ref = o64.cpu().numpy().ravel()
        got = omx.cpu().numpy().ravel()
        rel = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        fp64 = {"value": pts64 / (t64 * 1e-3) / 1e9, "unit": UNIT,
                "sample": "first 2 tracks, full grid, plain FP64 CUDA kernel",
                "mixed_speedup": value / ws / (pts64 / (t64 * 1e-3) / 1e9),
                "rel_l2_mixed_vs_fp64_cuda": rel}
        if rank == 0:
            accuracy = mixed_vs_oracle(w)

    # --- end to end through the public API, host tracks ---
    e2e = None
    if not args.no_e2e:
        n_e2e = args.e2e_steps or args.steps
        e2e_args = {"grid": w.args["grid"], "dtype": "mixed", "mode": mode}
        if not args.no_tune and args.shape is None:
            # the work shapes of the streamed chunks are tuned in the warm call
            e2e_args["autotune"] = min(args.tune_budget_ms, 3000.0)
        calc = SynchRad(e2e_args)
        host_tracks = [list(t) for t in w.tracks]
        calc.calculate_spectrum(host_tracks, timeStep=w.time_step, verbose=False,
                                L_screen=w.L_screen)  # warm (and tune)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            calc.calculate_spectrum(host_tracks, timeStep=w.time_step, verbose=False,
                                    L_screen=w.L_screen)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if dist:
            t = torch.tensor([el], device=device)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            el = float(t.item())
        e2e_spec = calc.Data["radiation"]["total"]
        host_ref = mixed_spec.cpu().numpy().swapaxes(-1, -3)
        # SynchRad strides the one workload over the ranks and sums on rank 0
        # (the reference's scheme): the whole job is pt_steps per call
        e2e = {"value": pt_steps * n_e2e / el / 1e9, "unit": UNIT,
               "scaling": "strong" if ws > 1 else "single GPU",
               "h2d_bytes_per_step": int(calc._h2d_bytes),
               "h2d": "tracks streamed in chunks on a copy stream, packed and copied "
                      "while the previous chunk computes",
               "d2h_bytes_per_step": int(P * 8),
               "steps": n_e2e, "ms_per_step": el / n_e2e * 1e3,
               "api": "SynchRad.calculate_spectrum (numpy tracks in, numpy spectrum out)",
               "matches_device_run": bool(np.allclose(e2e_spec, host_ref, rtol=1e-12, atol=0))}

    cpu = None
    if not args.no_cpu and rank == 0 and ws == 1:
        nth = os.cpu_count() or 1
        v, el, pts, kind = time_cpu_oracle(w, nth)
        cpu = {"value": v, "unit": UNIT, "cores": nth, "kind": kind,
               "sample": f"first 4 tracks on the full omega axis x 16 x 16 directions or "
                         f"screen points, FP64, {nth} threads, {el:.1f} s",
               "model": cpu_model(), "single_core": single_core_baseline(w, kind)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (mixed: double-float phase, compensated FP32 sums, FP64 spectrum)",
                "data": "synthetic",
                "config": {"workload": w.name, "n_tracks": len(w.tracks), "seed": args.seed,
                           "steps_per_track": (int(w.pt_steps // P // len(w.tracks)) + 1
                                               if args.workload != "ragged" else "500-20000"),
                           "grid": list(w.args["grid"][-1]),
                           "comp": "total", "pt_steps_per_step": pt_steps,
                           "l2": "flushed before every timed step (256 MB write, counted); "
                                 f"step records ({batch.total_steps * 64 / 1e6:.0f} MB) "
                                 + ("exceed L2" if batch.total_steps * 64 > 129e6
                                    else "fit in L2"),
                           "parallelism": f"replicas x{ws} (tracks independent)"},
                "e2e": e2e, "gpu_launches": 3 * args.steps,
                "launch": {"cuda_graph": graph is not None,
                           "graph_nodes": (dict(zip(("kernels", "nodes"), graph.nodes()))
                                           if graph is not None else None),
                           "shape": shape, "autotune": tune},
                "clocks": clk, "roofline": roofline, "cpu_baseline": cpu, "fp64_port": fp64,
                "accuracy": accuracy}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
