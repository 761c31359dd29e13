"""GPU parity: the CUDA path (through the C ABI) against the reference's own
outputs (golden fixtures) and the CPU oracle on the same seeded inputs.

Tolerances (stated per test):
  * deposition: 1e-12 relative to the grid maximum (bar: 1e-6);
  * interpolation, DF stage, history: 1e-10 relative to the field maximum;
  * plain FP64 wake: 1e-9 pointwise relative with a floor of 1e-3 of the peak
    (bar: 1e-4);
  * mixed-precision wake: max |a - b| / peak(|b|) <= 1e-4 and
    ||a - b|| / ||b|| <= 1e-4 over the mesh, peak and norm taken over both
    wake components (helpers.wake_errors); the pointwise error with a floor
    at 1e-3 of the peak is checked against 1e-2.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import (golden, oracle_from_wake_fixture, dep_from_array, lattice_from,
                           integ_from, rel_err, rms_rel, wake_errors, OracleRun)

pytestmark = pytest.mark.gpu

cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


def _maxrel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a - b)))


@cuda
def test_cic_golden_and_deterministic():
    from pydfcsr_gb300.deposit import histogram_cic_2d
    g = golden("cic.npz")
    nb1, lo1, hi1, nb2, lo2, hi2 = g["edge_grid"]
    out = histogram_cic_2d(g["edge_q1"], g["edge_q2"], g["edge_w"], int(nb1), lo1, hi1, int(nb2),
                           lo2, hi2)
    assert _maxrel(out, g["edge_out"]) < 1e-12
    gr = g["beam_grid"]
    args = (int(gr[0]), gr[1], gr[2], int(gr[3]), gr[4], gr[5])
    ones = histogram_cic_2d(g["beam_x"], g["beam_z"], np.ones(g["beam_x"].size), *args)
    pxw = histogram_cic_2d(g["beam_x"], g["beam_z"], g["beam_px"], *args)
    assert _maxrel(ones, g["beam_out_ones"]) < 1e-12
    assert _maxrel(pxw, g["beam_out_px"]) < 1e-12
    again = histogram_cic_2d(g["beam_x"], g["beam_z"], g["beam_px"], *args)
    assert np.array_equal(again, pxw), "deposit must be bitwise deterministic"


@cuda
@pytest.mark.parametrize("n,nb1,nb2", [(0, 16, 8), (1, 4, 4), (100_000, 128, 128),
                                       (1_000_000, 257, 100), (2_000_000, 512, 512)])
def test_cic_vs_oracle_sizes(n, nb1, nb2):
    from pydfcsr_gb300.deposit import deposit_cic
    rng = np.random.default_rng(n + nb1)
    x = rng.normal(0, 1e-5, n)
    z = rng.normal(0, 2e-5, n)
    w = rng.normal(0, 1e-5, n)
    g = (nb1, -4.5e-5, 4.5e-5, nb2, -9e-5, 9.5e-5)
    ref0 = O.histogram_cic_2d(x, z, np.ones(n), *g)
    ref1 = O.histogram_cic_2d(x, z, w, *g)
    dx, dz, dw = (torch.from_numpy(a).cuda() for a in (x, z, w))
    o0, o1 = deposit_cic(dx, dz, None, dw, *g)
    o0, o1 = o0.cpu().numpy(), o1.cpu().numpy()
    if n == 0:
        assert not o0.any() and not o1.any()
        return
    assert _maxrel(o0, ref0) < 1e-12
    assert _maxrel(o1, ref1) < 1e-12
    # mass conservation of the w=1 channel for particles inside the grid
    assert abs(o0.sum() - ref0.sum()) <= 1e-9 * max(ref0.sum(), 1)


@cuda
def test_interp_golden():
    from pydfcsr_gb300.interp3D import interpolate3D
    from pydfcsr_gb300.interp1D import interpolate1D
    g = golden("interp.npz")
    q = g["ka_small_q"]
    dx, dy, dz = g["ka_small_delta"]
    out = interpolate3D(q[:, 0], q[:, 1], q[:, 2], g["ka_small_data"], 1., 4., 7., dx, dy, dz)
    assert abs(out[0] - 125.80469388) < 5e-9
    np.testing.assert_array_equal(out, g["ka_small_out"])
    q = g["rnd_q"]
    out = interpolate3D(q[0], q[1], q[2], g["rnd_data"], *g["rnd_min"], *g["rnd_delta"])
    np.testing.assert_array_equal(out, g["rnd_out"])
    out = interpolate1D(g["i1_q"], g["i1_tab"], -2.0, 0.125)
    np.testing.assert_array_equal(out, g["i1_out"])


@cuda
@pytest.mark.parametrize("case", ["round", "tilt", "tilt1"])
def test_get_df_golden(case):
    from pydfcsr_gb300.deposit import DF_tracker
    g = golden("df.npz")
    dep = dep_from_array(g["params"])
    if case == "tilt1":
        dep["filter_order"] = 1
        dep["velocity_threhold"] = 5
    src = "tilt" if case == "tilt1" else case
    t = DF_tracker(dep)
    t.get_DF(g[src + "_x"], g[src + "_z"], g[src + "_px"], 0.25)
    for k in ("x_grids", "z_grids", "density", "vx", "density_x", "density_z", "vx_x"):
        ref = g[f"{case}_{k}"]
        out = getattr(t, k)
        assert out.shape == ref.shape, k
        if np.isnan(ref).all():
            assert np.isnan(out).all(), k
            continue
        assert _maxrel(out, ref) < 1e-10, (k, _maxrel(out, ref))


@cuda
def test_history_golden():
    from collections import OrderedDict
    from pydfcsr_gb300.harness import WakeRun
    g = golden("history.npz")
    lat = OrderedDict(step_size=0.01)
    lat["D1"] = {"type": "drift", "L": 0.08, "nsep": 1}
    run = WakeRun(lat, g["beam0"], dep_from_array(g["dep"]),
                  {"n_formation_length": 1.0, "zbins": 10, "xbins": 10},
                  {"xbins": 4, "zbins": 4, "xlim": 3, "zlim": 3}, precision="both")
    nsl = []
    for k in range(1, len(g["positions"])):
        run.coords = run.plan.matrix(k) @ run.coords
        run.beam.set_coords(run.coords)
        run.beam.position = float(run.plan.positions[k])
        run.csr.update_history(0.025)
        nsl.append(len(run.csr.DF_tracker.time_interp))
    np.testing.assert_array_equal(nsl, g["n_slices"])
    tr = run.csr.DF_tracker
    np.testing.assert_array_equal(np.array(tr.time_interp), g["h_time_interp"])
    for f in ("density", "density_x", "density_z", "vx", "vx_x"):
        ref = g["h_" + f]
        out = getattr(tr, f"data_{f}_interp")
        assert out.shape == ref.shape
        assert _maxrel(out, ref) < 1e-10, (f, _maxrel(out, ref))
    # FP32 ring holds the same fields rounded to float
    r = tr.ring
    idx = [(r.head + k) % r.cap for k in range(r.count)]
    f32 = r.ring32[idx][..., :5].double().cpu().numpy()
    f64 = r.ring64[idx].cpu().numpy()
    assert np.max(np.abs(f32 - f64)) <= 1e-7 * np.max(np.abs(f64))


def _device_run_from_fixture(g, precision="both"):
    from pydfcsr_gb300.harness import WakeRun
    mp = g["mesh_params"]
    mesh = {"xbins": int(mp[0]), "zbins": int(mp[1]), "xlim": float(mp[2]), "zlim": float(mp[3])}
    run = WakeRun(lattice_from(g), g["beam0"], dep_from_array(g["dep"]), integ_from(g), mesh,
                  precision=precision)
    for k in range(1, len(g["positions"])):
        run.step(k)
    return run


@cuda
@pytest.mark.parametrize("nx,nz,win,order", [(33, 47, 5, 2), (259, 31, 9, 1), (200, 130, 21, 3),
                                             (70, 300, 63, 2), (600, 40, 11, 2)])
def test_df_stage_shapes_vs_oracle(nx, nz, win, order):
    """The one-launch DF finalisation on grids that are not multiples of its
    32 x 32 smoothing tiles or 32-row trapz chunks, z lengths above one CTA,
    the longest window, against the oracle on the same particles: 1e-10 of
    each field's maximum (sums are evaluated in fixed orders of their own)."""
    from pydfcsr_gb300.deposit import DF_tracker
    from pydfcsr_gb300.synthetic import gaussian_beam
    b = gaussian_beam(40000, 10e-6, 20e-6, 1e-4, 5e-6, -8.0, seed=nx * 1000 + nz)
    dep = {"xbins": nx, "zbins": nz, "xlim": 5, "zlim": 5, "filter_order": order,
           "filter_window": win, "velocity_threhold": 1000}
    dev = DF_tracker(dep, grid_rule="configured")
    orc = O.DFTracker(dep, grid_rule="configured")
    dev.get_DF(b[0], b[4], b[1], 0.25)
    orc.get_DF(b[0], b[4], b[1], 0.25)
    for k in ("density", "vx", "density_x", "density_z", "vx_x"):
        out, ref = getattr(dev, k), getattr(orc, k)
        assert out.shape == ref.shape == (nx, nz), k
        assert _maxrel(out, ref) < 1e-10, (k, _maxrel(out, ref))


@cuda
@pytest.mark.parametrize("tag", ["dipole", "chicane_pos", "chicane_neg", "dipole_big"])
def test_wake_fp64_golden(tag):
    g = golden(f"wake_{tag}.npz")
    run = _device_run_from_fixture(g)
    csr = run.csr
    tr = csr.DF_tracker
    assert _maxrel(tr.data_density_interp, g["h_density"]) < 1e-10
    csr.get_CSR_mesh()
    np.testing.assert_allclose(csr.CSR_xmesh, g["xmesh"], rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(csr.CSR_zmesh, g["zmesh"], rtol=1e-12, atol=1e-18)
    # the device mesh is the host mesh bit for bit
    sd, xd = csr.mesh_device()
    assert np.array_equal(sd.cpu().numpy(), run.beam.position + csr.CSR_zmesh)
    assert np.array_equal(xd.cpu().numpy(), csr.CSR_xmesh)
    s = run.beam.position + g["zmesh"][g["points"]]
    x = g["xmesh"][g["points"]]
    dE, xk = csr.wake_device(torch.from_numpy(s).cuda(), torch.from_numpy(x).cuda(), "fp64")
    assert rel_err(dE.cpu().numpy(), g["wake_dE"]) < 1e-9
    assert rel_err(xk.cpu().numpy(), g["wake_xkick"]) < 1e-9
    if "mesh_dE" in g.files:
        csr.calculate_2D_CSR("fp64")
        assert rel_err(csr.dE_dct, g["mesh_dE"]) < 1e-9
        assert rel_err(csr.x_kick, g["mesh_xkick"]) < 1e-9
        # mixed precision on the same history: max_rel, rms_rel and the
        # pointwise error (floor 1e-3 of the peak) all <= 1e-4
        csr.calculate_2D_CSR("mixed")
        e = wake_errors(csr.dE_dct, csr.x_kick, g["mesh_dE"], g["mesh_xkick"])
        assert max(e.values()) <= 1e-4, e


@cuda
@pytest.mark.parametrize("tag", ["dipole", "chicane_pos"])
def test_wake_mixed_geometry_paths(tag):
    """The mixed kernel's two geometry paths on the same history: with the
    double-word orbit tables (the default) and without them (FP64 geometry,
    for C-ABI callers that leave the tables out).  Each is within 1e-4 of
    the reference's mesh wake, and the two agree to 1e-6 of the peak."""
    from pydfcsr_gb300.CSR import jobs_to_device
    g = golden(f"wake_{tag}.npz")
    run = _device_run_from_fixture(g)
    csr = run.csr
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    ip = csr.integration_params
    out = {}
    for path in ("dw", "fp64"):
        job = csr._job()
        if path == "fp64":
            job.lattice_dw = None
            job.lattice_delta_dw = None
        dE, xk = csr.evaluator.mixed(jobs_to_device([job]), s, x, ip.xbins, ip.zbins)
        out[path] = (dE.cpu().numpy(), xk.cpu().numpy())
    for path, (dE, xk) in out.items():
        e = wake_errors(dE, xk, g["mesh_dE"], g["mesh_xkick"])
        assert max(e.values()) <= 1e-4, (path, e)
    e = wake_errors(*out["fp64"], *out["dw"])
    assert e["max_rel"] < 1e-6, e
    # the same job passed by value (dfcsr_wake_mixed_job, what wake_device
    # uses) gives the device-job result bit for bit
    dE, xk = csr.evaluator.mixed_job(csr._job(), s, x, ip.xbins, ip.zbins)
    assert np.array_equal(dE.cpu().numpy(), out["dw"][0])
    assert np.array_equal(xk.cpu().numpy(), out["dw"][1])


@cuda
def test_wake_fp64_bitwise_on_oracle_history():
    """Same history, same beam statistics: the FP64 kernel reproduces the
    oracle (and so the reference) exactly."""
    g = golden("wake_dipole.npz")
    orc = oracle_from_wake_fixture(g)
    run = _device_run_from_fixture(g, precision="fp64")
    tr = run.csr.DF_tracker
    # overwrite the device ring with the oracle's history
    r = tr.ring
    data = np.stack([orc.tracker.data_density_interp, orc.tracker.data_density_x_interp,
                     orc.tracker.data_density_z_interp, orc.tracker.data_vx_interp,
                     orc.tracker.data_vx_x_interp], axis=-1)
    assert data.shape[0] == r.count
    for k in range(r.count):
        r.ring64[(r.head + k) % r.cap].copy_(torch.from_numpy(np.ascontiguousarray(data[k])))
    for a in ("min_x", "min_y", "min_z", "delta_x", "delta_y", "delta_z"):
        setattr(tr, a, getattr(orc.tracker, a))
    st = orc.stats()
    b = run.beam
    b._sigma_x, b._sigma_z, b._mean_x = st["sigma_x"], st["sigma_z"], st["mean_x"]
    b._slope = st["slope"]
    run.csr.formation_length = orc.lf
    w = orc.wake_oracle()
    pts = g["points"]
    s = orc.position + g["zmesh"][pts]
    x = g["xmesh"][pts]
    ref = w.points(s, x)
    dE, xk = run.csr.wake_device(torch.from_numpy(s).cuda(), torch.from_numpy(x).cuda(), "fp64")
    np.testing.assert_array_equal(dE.cpu().numpy(), ref[0])
    np.testing.assert_array_equal(xk.cpu().numpy(), ref[1])
    # more s' columns than the kernel's static shared memory holds (1024):
    # the column sums go to dynamic shared memory, still bit for bit
    zb = 1536
    run.csr.integration_params.zbins = zb
    w2 = O.WakeOracle(orc.tracker, orc.tables, orc.position, st["sigma_z"], st["sigma_x"],
                      st["slope"][0], st["mean_x"], orc.lf, orc.integ["n_formation_length"], zb,
                      orc.integ["xbins"], charge=orc.charge)
    ref2 = w2.points(s[:2], x[:2])
    dE2, xk2 = run.csr.wake_device(torch.from_numpy(s[:2]).cuda(), torch.from_numpy(x[:2]).cuda(),
                                   "fp64")
    np.testing.assert_array_equal(dE2.cpu().numpy(), ref2[0])
    np.testing.assert_array_equal(xk2.cpu().numpy(), ref2[1])


@cuda
def test_wake_mixed_at_maximum_integration_bins():
    """The mixed wake at its largest integration grid: 512 x' bins (the far
    region's 1024 rows staged in shared memory) and 4096 s' bins (32 column
    chunks per region), against the FP64 kernel with the same bins on three
    observation points: max_rel, rms_rel and pointwise <= 1e-4."""
    g = golden("wake_dipole.npz")
    run = _device_run_from_fixture(g)
    csr = run.csr
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    idx = torch.tensor([0, s.numel() // 2 + 7, s.numel() - 3], device="cuda")
    s3, x3 = s[idx].contiguous(), x[idx].contiguous()
    ip = csr.integration_params
    ip.xbins, ip.zbins = 512, 4096
    dE64, xk64 = csr.wake_device(s3, x3, "fp64")
    dE, xk = csr.wake_device(s3, x3, "mixed")
    ref = (dE64.cpu().numpy(), xk64.cpu().numpy())
    assert np.isfinite(ref[0]).all() and np.isfinite(ref[1]).all()
    e = wake_errors(dE.cpu().numpy(), xk.cpu().numpy(), *ref)
    assert max(e.values()) <= 1e-4, e


@cuda
def test_wake_integrand_debug_golden():
    g = golden("wake_dipole.npz")
    run = _device_run_from_fixture(g, precision="fp64")
    csr = run.csr
    i = g["points"][0]
    dbg = csr.get_CSR_wake(run.beam.position + g["zmesh"][i], g["xmesh"][i], debug=True)
    nb = int(g["debug_n"])
    assert len(dbg) == nb
    for j in range(nb):
        ref = g[f"debug_{j}"]
        assert np.shape(dbg[j]) == ref.shape
        assert _maxrel(dbg[j], ref) < 1e-9, j


@cuda
def test_wake_chicane_mixed_vs_oracle():
    """C2-shaped chicane (reduced N, full grid sizes) at a step in the
    4-region chirped branch: mixed-precision wake within 1e-4 of the oracle."""
    from pydfcsr_gb300.synthetic import workload
    from pydfcsr_gb300.harness import WakeRun
    wl = workload("chicane_c2", n_particles=200_000)
    mesh = {"xbins": 8, "zbins": 8, "xlim": 3, "zlim": 3}
    orc = OracleRun(wl.lattice, wl.beam(), wl.deposit, wl.integration, grid_rule="configured")
    run = WakeRun(wl.lattice, wl.beam(), wl.deposit, wl.integration, mesh, precision="both",
                  grid_rule="configured")
    orc.init()
    steps = 40
    for k in range(1, steps + 1):
        orc.step(k)
        run.step(k)
    assert abs(orc.stats()["slope"][0]) > 1.0
    st = orc.stats()
    xm, zm, _, _ = O.csr_mesh(st, 8, 8, 3, 3)
    ref = orc.wake_oracle().points(orc.position + zm, xm, nthreads=8)
    dE64, xk64 = run.wake("fp64")
    dE32, xk32 = run.wake("mixed")
    assert rel_err(dE64.ravel(), ref[0]) < 1e-8
    assert rel_err(xk64.ravel(), ref[1]) < 1e-8
    e = wake_errors(dE32, xk32, ref[0], ref[1])
    assert max(e.values()) <= 1e-4, e


@cuda
def test_rgi_axis_tables_on_device_equal_host():
    """dfcsr_rgi_axis_linspace == the RegularGridInterpolator tables computed
    from the numpy linspace arrays (bit for bit), including targets outside
    the source grid on both sides and targets on source points."""
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.coeffs import rgi_axis
    from pydfcsr_gb300.runtime import ptr, stream_handle
    cases = [((-1.0e-4, 1.0e-4, 256), (-1.3e-4, 1.3e-4, 500)),
             ((2.0, 3.0, 11), (2.0, 3.0, 11)),
             ((2.0, 3.0, 11), (2.0, 3.0, 21)),
             ((-5e-5, 7e-5, 128), (-2e-5, 2e-5, 600)),
             ((0.0, 1.0, 2), (-0.5, 1.5, 9))]
    for (s0, s1, ns), (t0, t1, nt) in cases:
        i_ref, w_ref, o_ref = rgi_axis(np.linspace(s0, s1, ns), np.linspace(t0, t1, nt))
        idx = torch.empty(nt, dtype=torch.int32, device="cuda")
        w = torch.empty(nt, dtype=torch.float64, device="cuda")
        o = torch.empty(nt, dtype=torch.uint8, device="cuda")
        _lib.call("dfcsr_rgi_axis_linspace", s0, s1, ns, t0, t1, nt, ptr(idx), ptr(w), ptr(o),
                  stream_handle())
        assert np.array_equal(idx.cpu().numpy(), i_ref)
        assert np.array_equal(w.cpu().numpy(), w_ref)
        assert np.array_equal(o.cpu().numpy(), o_ref)


@cuda
def test_calculate_2d_csr_nonblocking_matches_blocking():
    """calculate_2D_CSR(wait=False) gives the same arrays as the blocking call,
    through the returned handle and through the dE_dct / x_kick attributes."""
    g = golden("wake_dipole.npz")
    run = _device_run_from_fixture(g, precision="both")
    csr = run.csr
    csr.get_CSR_mesh()
    csr.calculate_2D_CSR("mixed")
    dE0, xk0 = csr.dE_dct.copy(), csr.x_kick.copy()
    pend = csr.calculate_2D_CSR("mixed", wait=False)
    dE1, xk1 = pend.result()
    assert np.array_equal(dE0, dE1) and np.array_equal(xk0, xk1)
    csr.calculate_2D_CSR("mixed", wait=False)
    assert np.array_equal(csr.dE_dct, dE0) and np.array_equal(csr.x_kick, xk0)
    # the library's launch counter sees the mesh kernel and the wake's job
    # store, set-up, geometry, integral and finalize launches (one batch here)
    from pydfcsr_gb300 import _lib
    n0 = _lib.kernel_launches()
    csr.calculate_2D_CSR("mixed")
    assert _lib.kernel_launches() - n0 == 6


@cuda
@pytest.mark.parametrize("x0,x1,nx,z0,z1,nz", [
    (0.0, 1.0, 5, -2.0, 2.0, 9),                    # exact spacings: numpy's uniform branch
    (-1.07e-4, 1.31e-4, 256, -2.6e-4, 2.2e-4, 256),  # spacings that differ by an ulp
    (3.3e-5, 9.1e-5, 2, -5e-5, 5e-5, 513),
])
def test_df_axis_tables_match_numpy(x0, x1, nx, z0, z1, nz):
    """dfcsr_df_axis_tables against coeffs.gradient_table (numpy.gradient's
    coefficients) and numpy.diff on the host's linspace grids: bit for bit."""
    import ctypes
    import torch
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.coeffs import gradient_table
    from pydfcsr_gb300.runtime import stream_handle
    xg, zg = np.linspace(x0, x1, nx), np.linspace(z0, z1, nz)
    gxh, gxu, _ = gradient_table(xg)
    gzh, gzu, _ = gradient_table(zg)
    gx = torch.full((4, nx), np.nan, dtype=torch.float64, device="cuda")
    gz = torch.full((4, nz), np.nan, dtype=torch.float64, device="cuda")
    dx = torch.full((max(nx - 1, 1),), np.nan, dtype=torch.float64, device="cuda")
    dz = torch.full((nz - 1,), np.nan, dtype=torch.float64, device="cuda")
    _lib.call("dfcsr_df_axis_tables", x0, x1, nx, z0, z1, nz, int(gxu), int(gzu),
              ctypes.c_void_p(gx.data_ptr()), ctypes.c_void_p(gz.data_ptr()),
              ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dz.data_ptr()), stream_handle())
    assert np.array_equal(gx.cpu().numpy(), gxh)
    assert np.array_equal(gz.cpu().numpy(), gzh)
    assert np.array_equal(dx.cpu().numpy()[:nx - 1], np.diff(xg))
    assert np.array_equal(dz.cpu().numpy(), np.diff(zg))
