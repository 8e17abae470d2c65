"""The C ABI used from a plain C program (tests/c_abi/sr_c_example.c).

The program includes only include/synchrad_gb300.h and the CUDA runtime
header, allocates its device buffers with cudaMalloc and evaluates one
far-field 'total' spectrum with SR_PREC_MIXED and SR_PREC_DOUBLE; the GPU test
compares both with the oracle on the same seeded track (the reference's
`total` kernel, synchrad/kernel_farfield.cl:6, restated in C)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "c_abi" / "sr_c_example.c"
CUDA_HOME = Path("/usr/local/cuda")


def build_program(out_dir: Path) -> Path:
    """Compiles and links the example against the in-tree library."""
    if shutil.which("gcc") is None or not (CUDA_HOME / "include" / "cuda_runtime_api.h").exists():
        pytest.skip("gcc or the CUDA runtime headers are missing")
    from synchrad_gb300 import _lib
    lib = Path(_lib.lib_path())
    exe = out_dir / "sr_c_example"
    cuda_lib = next((p for p in (CUDA_HOME / "lib64", CUDA_HOME / "lib")
                     if (p / "libcudart.so").exists()), CUDA_HOME / "lib64")
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-O2",
           f"-I{ROOT / 'include'}", f"-I{CUDA_HOME / 'include'}", str(SRC), "-o", str(exe),
           f"-L{lib.parent}", "-lsynchrad_gb300", f"-L{cuda_lib}", "-lcudart",
           f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{cuda_lib}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def make_problem(seed=7):
    from synchrad_gb300 import workloads as wl
    tracks, dt, k_res = wl.analytic_undulator_tracks(
        n_particles=1, n_periods=6, steps_per_period=24, seed=seed)
    track6 = [np.ascontiguousarray(a, dtype=np.float64) for a in tracks[0][:6]]
    omega = 2 * np.pi * np.linspace(0.05 * k_res, 1.2 * k_res, 48)
    theta = np.linspace(0.0, 0.02, 6)
    phi = np.linspace(0.0, 2 * np.pi, 5)
    axes = [np.ascontiguousarray(v) for v in
            (omega, np.sin(theta), np.cos(theta), np.sin(phi), np.cos(phi))]
    return track6, axes, dt, 1.3


def write_input(path: Path, track6, axes, dt, weight):
    n = track6[0].size
    with open(path, "wb") as f:
        f.write(np.array([n, axes[0].size, axes[1].size, axes[3].size], "<u4").tobytes())
        f.write(np.array([dt, weight], "<f8").tobytes())
        for a in list(track6) + list(axes):
            f.write(np.asarray(a, "<f8").tobytes())


def test_c_program_compiles_and_links(tmp_path):
    exe = build_program(tmp_path)
    assert exe.exists()
    out = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True,
                         check=True).stdout
    for name in ("sr_spectrum", "sr_workspace_bytes", "sr_workspace_status", "sr_last_error"):
        assert name in out


@pytest.mark.gpu
def test_c_program_matches_oracle(tmp_path):
    import oracle
    exe = build_program(tmp_path)
    track6, axes, dt, weight = make_problem()
    write_input(tmp_path / "in.bin", track6, axes, dt, weight)
    run = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                         capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    nO, nT, nP = axes[0].size, axes[1].size, axes[3].size
    got = np.fromfile(tmp_path / "out.bin", "<f8").reshape(2, nP, nT, nO)

    n = track6[0].size
    ref = np.zeros((1, nP, nT, nO))
    oracle.run_track("port", "far", "total", [ref], track6, weight, 0, n, n, axes,
                     (nO, nT, nP), dt, np.array([n], np.uint32))
    ref = ref[0]
    scale = np.linalg.norm(ref)
    assert scale > 0
    # mixed precision: relative L2 within 1e-5 of the FP64 oracle
    assert np.linalg.norm(got[0] - ref) / scale < 1e-5
    # the FP64 kernel follows the oracle to rounding
    assert np.linalg.norm(got[1] - ref) / scale < 1e-12
