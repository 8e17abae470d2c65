"""GPU parity: the CUDA library against the golden vectors of the reference.

Tolerances (relative L2 over all output arrays of a comp, and per array for
arrays carrying more than 1e-6 of the comp's norm):
  * dtype 'double' (plain FP64 kernel): 1e-12.  Same IEEE operation order as
    the reference (no contraction); only sin/cos differ in the last bit.
  * dtype 'float' (FP32 kernel): 1e-5.  Phases are computed identically; the
    FP32 sin/cos of the GPU and of glibc differ by an ulp or two.
  * dtype 'mixed' against the FP64 golden vectors: 1e-5 (the target accuracy
    of the mixed-precision path).
  * dtype 'double-float' (far field) against the FP64 golden vectors: 1e-10
    (about 48-bit arithmetic; the reference's own FP64 phase carries ~1e-9 rad
    at the largest phases, which averages down in the sums).
"""
import ctypes

import numpy as np
import pytest

import golden_cases as gc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"double": 1e-12, "float": 1e-5, "mixed": 1e-5, "double-float": 1e-10}


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def run_case(case, dtype=None):
    from synchrad_gb300.calc import SynchRad
    args = case.fresh_args()
    if dtype is not None:
        args["dtype"] = dtype
    calc = SynchRad(args)
    if case.omega is not None:
        # evaluate on the fixture's own omega axis (a log-spaced axis is built
        # with np.exp, whose last bit differs between platforms)
        calc.Args["omega"] = np.asarray(case.omega).astype(calc.dtype)
        calc._init_data()
    calc.calculate_spectrum(case.fresh_tracks(), verbose=False, **case.call)
    return calc


def compare(got: dict, exp: dict, tol: float, name=""):
    keys = sorted(exp)
    e_all = np.concatenate([exp[k].ravel() for k in keys])
    g_all = np.concatenate([got[k].ravel() for k in keys])
    assert g_all.shape == e_all.shape, name
    assert np.all(np.isfinite(g_all)), name
    norm = np.linalg.norm(e_all)
    if norm == 0:
        assert np.all(g_all == 0), name
        return 0.0
    rel = np.linalg.norm(g_all - e_all) / norm
    assert rel <= tol, f"{name}: relative L2 {rel:.3e} > {tol:.1e}"
    for k in keys:
        nk = np.linalg.norm(exp[k])
        if nk > 1e-6 * norm:
            rk = np.linalg.norm(got[k] - exp[k]) / nk
            assert rk <= 10 * tol, f"{name}[{k}]: relative L2 {rk:.3e}"
    return rel


@pytest.mark.parametrize("name", gc.names())
def test_golden_native_dtype(name):
    """Each golden case in its own dtype ('double' or 'float')."""
    _need_gpu()
    case = gc.load(name)
    calc = run_case(case)
    compare(calc.Data["radiation"], case.expected, TOL[case.args.get("dtype", "double")], name)
    assert calc.total_weight == pytest.approx(case.total_weight, rel=1e-12)
    assert np.array_equal(np.asarray(calc.snap_iterations), case.snap_iterations)


@pytest.mark.parametrize("name", [n for n in gc.names()
                                  if n.startswith("far_") and not n.endswith("_float")])
def test_golden_mixed_far(name):
    """Mixed precision against the FP64 reference on every far-field case."""
    _need_gpu()
    case = gc.load(name)
    calc = run_case(case, dtype="mixed")
    compare(calc.Data["radiation"], case.expected, TOL["mixed"], name)


@pytest.mark.parametrize("name", [n for n in gc.names()
                                  if n.startswith("near_") and not n.endswith("_float")])
def test_golden_mixed_near(name):
    """Mixed precision against the FP64 reference on every near-field case."""
    _need_gpu()
    case = gc.load(name)
    calc = run_case(case, dtype="mixed")
    compare(calc.Data["radiation"], case.expected, TOL["mixed"], name)


@pytest.mark.parametrize("name", [n for n in gc.names()
                                  if n.startswith("far_") and not n.endswith("_float")])
def test_golden_double_float_far(name):
    """Double-float arithmetic against the FP64 reference on every far-field case."""
    _need_gpu()
    case = gc.load(name)
    calc = run_case(case, dtype="double-float")
    rel = compare(calc.Data["radiation"], case.expected, TOL["double-float"], name)
    print(f"{name}: double-float relative L2 {rel:.2e}")


@pytest.mark.parametrize("K", [8, 16])
@pytest.mark.parametrize("name", [n for n in gc.names()
                                  if n.startswith("near_") and not n.endswith("_float")])
def test_golden_mixed_near_points_per_lane(name, K):
    """Both near-field work shapes (8 and 16 omega points per lane) on every
    near-field case: the shape is pinned for the case's sizes before the call."""
    _need_gpu()
    from synchrad_gb300 import _lib
    from synchrad_gb300 import batch as bt
    from synchrad_gb300.calc import VEC_COMPS
    case = gc.load(name)
    calc = run_case(case, dtype="mixed")  # the grid and the batch sizes of the call
    it_range = case.call.get("it_range")
    n_snaps = int(case.call.get("nSnaps", 1))
    batch = bt.pack_tracks(case.fresh_tracks(), np.float64, n_snaps, case.call["timeStep"],
                           it_range=it_range, device="cuda")
    comp = case.call.get("comp", "total")
    L = 32
    while L > 8 and (L // 2) * K >= int(calc.Args["gridNodeNums"][0]):
        L //= 2
    try:
        bt.set_config(batch, calc._grid_dev, comp, _lib.SR_PREC_MIXED, points_per_lane=K,
                      lanes_per_direction=L)
        assert bt.current_config(batch, calc._grid_dev, comp)["points_per_lane"] == K
        calc2 = run_case(case, dtype="mixed")
        assert sorted(calc2.Data["radiation"]) == sorted(VEC_COMPS[comp])
        compare(calc2.Data["radiation"], case.expected, TOL["mixed"], f"{name} K={K}")
    finally:
        _lib.lib().sr_config_clear()


def test_mixed_is_deterministic():
    _need_gpu()
    case = gc.load("far_total_ragged_wmean")
    a = run_case(case, dtype="mixed").Data["radiation"]["total"]
    b = run_case(case, dtype="mixed").Data["radiation"]["total"]
    assert np.array_equal(a, b)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", ["far_total_double", "far_cartesian_complex_double",
                                  "near_cartesian_double", "far_spheric_float"])
def test_per_track_entry_points(name):
    """The reference's kernel argument lists through the C ABI, one call per track."""
    _need_gpu()
    from synchrad_gb300 import _lib
    from oracle import host
    L = _lib.lib()
    case = gc.load(name)
    a = host.init_args(case.fresh_args())
    dt_np = np.float64 if a["dtype"] == "double" else np.float32
    axes = [_dev(v) for v in host.device_axes(a)]
    comp = case.call["comp"]
    keys = host.VEC_COMPS[comp]
    n_snaps = int(case.call.get("nSnaps", 1))
    shape = (n_snaps,) + tuple(a["gridNodeNums"][::-1])
    spectra = [torch.zeros(shape, dtype=torch.float64 if dt_np == np.float64 else torch.float32,
                           device="cuda") for _ in keys]
    ff = _dev(host.form_factor(a, case.call.get("sigma_particle", 0)))
    step = dt_np(case.call["timeStep"])
    fn = getattr(L, {("far", "total"): "sr_far_total",
                     ("far", "cartesian"): "sr_far_cartesian_comps",
                     ("far", "cartesian_complex"): "sr_far_cartesian_comps_complex",
                     ("far", "spheric"): "sr_far_spheric_comps",
                     ("far", "spheric_complex"): "sr_far_spheric_comps_complex",
                     ("near", "total"): "sr_near_total",
                     ("near", "cartesian"): "sr_near_cartesian_comps",
                     ("near", "cartesian_complex"): "sr_near_cartesian_comps_complex"}
                 [(a["mode"], comp)])
    dtype_id = 0 if dt_np == np.float64 else 1
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for tr in case.fresh_tracks():
        coords = [_dev(np.asarray(v, dtype=dt_np)) for v in tr[:6]]
        n = coords[0].numel()
        snaps = _dev(host.snap_iterations((0, n), n_snaps).view(np.int32))
        args = [dtype_id, 0] + [s.data_ptr() for s in spectra] + [c.data_ptr() for c in coords]
        args += [float(dt_np(tr[6])), 0, n, n]
        if a["mode"] == "far":
            args += [t.data_ptr() for t in axes] + list(map(int, a["gridNodeNums"]))
        else:
            args += [t.data_ptr() for t in axes] + [float(dt_np(case.call["L_screen"]))]
            args += list(map(int, a["gridNodeNums"]))
        args += [float(step), n_snaps, snaps.data_ptr()]
        if comp.endswith("complex"):
            args.append(ff.data_ptr())
        args.append(stream)
        _lib.check(fn(*args))
    torch.cuda.synchronize()
    got = {k: np.ascontiguousarray(s.cpu().numpy().swapaxes(-1, -3), dtype=np.double)
           for k, s in zip(keys, spectra)}
    compare(got, case.expected, TOL[a["dtype"]], name)


def test_invalid_arguments_raise():
    _need_gpu()
    from synchrad_gb300 import _lib
    L = _lib.lib()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    sp = torch.zeros(8, dtype=torch.float64, device="cuda")
    snaps = torch.tensor([4], dtype=torch.int32, device="cuda")
    p = x.data_ptr()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.sr_far_total(0, 0, sp.data_ptr(), p, p, p, p, p, p, 1.0, 0, 0, 4, p, p, p, p, p,
                        2, 2, 2, 0.1, 1, snaps.data_ptr(), stream)
    assert rc == _lib.SR_ERR_INVALID
    assert b"itEnd" in L.sr_last_error()
    rc = L.sr_far_total(7, 0, sp.data_ptr(), p, p, p, p, p, p, 1.0, 0, 4, 4, p, p, p, p, p,
                        2, 2, 2, 0.1, 1, snaps.data_ptr(), stream)
    assert rc == _lib.SR_ERR_INVALID


def test_accumulates_across_calls():
    """Two calls on the same arrays add up, as repeated kernel launches do."""
    _need_gpu()
    from synchrad_gb300.batch import make_grid, pack_tracks, run_spectrum
    from oracle import host
    case = gc.load("far_total_double")
    a = host.init_args(case.fresh_args())
    grid = make_grid("far", host.device_axes(a), a["gridNodeNums"], torch.float64, "cuda")
    batch = pack_tracks(case.fresh_tracks(), np.float64, 1, case.call["timeStep"], device="cuda")
    out = torch.zeros((1,) + tuple(a["gridNodeNums"][::-1]), dtype=torch.float64, device="cuda")
    for prec in (0, 3):
        out.zero_()
        run_spectrum(batch, grid, "total", prec, [out], check_status=True)
        once = out.clone()
        run_spectrum(batch, grid, "total", prec, [out], check_status=True)
        torch.cuda.synchronize()
        assert torch.allclose(out, 2 * once, rtol=1e-14, atol=0)
