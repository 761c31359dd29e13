"""Pin the CPU oracle against fixtures produced by running the reference itself.

The fixtures (``tests/golden/*.npz``) come from ``tests/golden/make_golden.py``
which imports pyDFCSR_2D and calls its own functions.  The C restatement of
the numba loops and of the wake integral reproduces the reference's IEEE
arithmetic in the same order, so those comparisons are exact or within a few
ulps; the scipy restatements (Savitzky-Golay, RegularGridInterpolator) agree
to ~1e-13 relative.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import golden, oracle_from_wake_fixture, dep_from_array, rel_err
from pydfcsr_gb300.synthetic import StepPlan


def test_interp3d_known_answer():
    g = golden("interp.npz")
    d = g["ka_small_data"]
    q = g["ka_small_q"]
    dx, dy, dz = g["ka_small_delta"]
    out = O.interpolate3D(q[:, 0], q[:, 1], q[:, 2], d, 1., 4., 7., dx, dy, dz)
    # scipy RegularGridInterpolator on the same grid, recorded in
    # test/test_interpolation.ipynb: 125.80469388
    assert abs(out[0] - 125.80469388) < 5e-9
    np.testing.assert_array_equal(out, g["ka_small_out"])


def test_interp3d_notebook_grid():
    g = golden("interp.npz")
    x = np.linspace(1, 4, 200); y = np.linspace(4, 7, 200); z = np.linspace(7, 9, 100)
    xg, yg, zg = np.meshgrid(x, y, z, indexing="ij")
    d = 2 * xg ** 3 + 3 * yg ** 2 - zg
    dx, dy, dz = g["ka_big_delta"]
    out = O.interpolate3D([2.1], [6.2], [8.3], d, 1., 4., 7., dx, dy, dz)
    np.testing.assert_array_equal(out, g["ka_big_out"])


def test_interp3d_random_and_edges():
    g = golden("interp.npz")
    q = g["rnd_q"]
    out = O.interpolate3D(q[0], q[1], q[2], g["rnd_data"], *g["rnd_min"], *g["rnd_delta"])
    np.testing.assert_array_equal(out, g["rnd_out"])
    # the (-1, 0) band extrapolates, so some of those outputs are nonzero
    u = (q - g["rnd_min"][:, None]) / g["rnd_delta"][:, None]
    band = np.any((u > -1) & (u < 0), axis=0) & np.all(u > -1, axis=0) & \
        np.all(u < np.array([[7], [9], [12]]), axis=0)
    assert np.count_nonzero(out[band]) > 10


def test_interp1d():
    g = golden("interp.npz")
    out = O.interpolate1D(g["i1_q"], g["i1_tab"], -2.0, 0.125)
    np.testing.assert_array_equal(out, g["i1_out"])


def test_cic_edges_exact():
    g = golden("cic.npz")
    nb1, lo1, hi1, nb2, lo2, hi2 = g["edge_grid"]
    out = O.histogram_cic_2d(g["edge_q1"], g["edge_q2"], g["edge_w"], int(nb1), lo1, hi1,
                             int(nb2), lo2, hi2)
    np.testing.assert_array_equal(out, g["edge_out"])


def test_cic_beam_exact():
    g = golden("cic.npz")
    gr = g["beam_grid"]
    args = (int(gr[0]), gr[1], gr[2], int(gr[3]), gr[4], gr[5])
    ones = O.histogram_cic_2d(g["beam_x"], g["beam_z"], np.ones(g["beam_x"].size), *args)
    pxw = O.histogram_cic_2d(g["beam_x"], g["beam_z"], g["beam_px"], *args)
    np.testing.assert_array_equal(ones, g["beam_out_ones"])
    np.testing.assert_array_equal(pxw, g["beam_out_px"])


@pytest.mark.parametrize("window,order", [(5, 1), (5, 2), (9, 1), (9, 2), (7, 3), (11, 2)])
def test_savgol_matches_scipy(window, order):
    scipy_signal = pytest.importorskip("scipy.signal")
    rng = np.random.default_rng(window * 10 + order)
    a = rng.normal(size=(23, 31)) + np.linspace(0, 5, 31)
    for axis in (0, 1):
        ref = scipy_signal.savgol_filter(a, window, order, axis=axis)
        out = O.savgol_filter(a, window, order, axis)
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12)


def test_gradient_matches_numpy():
    rng = np.random.default_rng(3)
    f = rng.normal(size=(17, 29))
    xg = np.linspace(-3e-5, 4e-5, 17)
    zg = np.linspace(1e-4, 3e-4, 29)
    fx, fz = O.gradient2d(f, xg, zg)
    rx, rz = np.gradient(f, xg, zg)
    np.testing.assert_array_equal(fx, rx)
    np.testing.assert_array_equal(fz, rz)


def test_rgi_matches_scipy():
    interp = pytest.importorskip("scipy.interpolate")
    rng = np.random.default_rng(5)
    xg = np.linspace(-1.3, 2.1, 23)
    zg = np.linspace(0.2, 0.9, 17)
    v = rng.normal(size=(23, 17))
    X, Z = np.meshgrid(np.linspace(-1.6, 2.4, 41), np.linspace(0.1, 1.0, 37), indexing="ij")
    ref = interp.RegularGridInterpolator((xg, zg), v, method="linear", fill_value=0.25,
                                         bounds_error=False)((X, Z))
    out = O.rgi_linear_2d(xg, zg, v, X, Z, 0.25)
    np.testing.assert_allclose(out, ref, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("case", ["round", "tilt", "tilt1"])
def test_get_df(case):
    g = golden("df.npz")
    p = g["params"]
    dep = dep_from_array(p)
    if case == "tilt1":
        dep["filter_order"] = 1
        dep["velocity_threhold"] = 5
    src = "tilt" if case == "tilt1" else case
    t = O.DFTracker(dep)
    t.get_DF(g[src + "_x"], g[src + "_z"], g[src + "_px"], 0.25)
    for k in ("x_grids", "z_grids", "density", "vx", "density_x", "density_z", "vx_x"):
        ref = g[f"{case}_{k}"]
        out = getattr(t, k)
        assert out.shape == ref.shape, k
        if np.isnan(ref).all():
            assert np.isnan(out).all(), k
            continue
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(out - ref)) <= 1e-11 * scale, (k, np.max(np.abs(out - ref)) / scale)


def test_lattice_tables():
    g = golden("lattice.npz")
    for tag in ("dipole", "chicane"):
        el = g[tag + "_elements"]
        from collections import OrderedDict
        lat = OrderedDict(step_size=0.1)
        for i, (L, ang, dip) in enumerate(el):
            lat[f"e{i}"] = ({"type": "dipole", "L": L, "angle": ang, "nsep": 1} if dip
                            else {"type": "drift", "L": L, "nsep": 1})
        s, rho, dist, nsep, coords, nv, tau = O.reference_trajectory(lat, 2000)
        np.testing.assert_array_equal(s, g[tag + "_s"])
        np.testing.assert_array_equal(rho, g[tag + "_rho"])
        np.testing.assert_array_equal(dist, g[tag + "_distance"])
        np.testing.assert_array_equal(coords, g[tag + "_coords"])
        np.testing.assert_array_equal(nv, g[tag + "_n_vec"])
        np.testing.assert_array_equal(tau, g[tag + "_tau_vec"])


def test_history_sequence():
    from collections import OrderedDict
    from tests.helpers import OracleRun
    g = golden("history.npz")
    lat = OrderedDict(step_size=0.01)
    lat["D1"] = {"type": "drift", "L": 0.08, "nsep": 1}
    run = OracleRun(lat, g["beam0"], dep_from_array(g["dep"]),
                    {"n_formation_length": 1.0, "zbins": 10, "xbins": 10})
    run.init()
    nsl = []
    for k in range(1, len(g["positions"])):
        run.beam6 = run.plan.matrix(k) @ run.beam6
        run.position = run.plan.positions[k]
        run.df_step(0.025)
        run.tracker.build_interpolant()
        nsl.append(len(run.tracker.time_interp))
    np.testing.assert_array_equal(nsl, g["n_slices"])
    tr = run.tracker
    np.testing.assert_array_equal(np.array(tr.time_interp), g["h_time_interp"])
    for a, b in (("min_x", "t_min"), ("delta_x", "t_delta"), ("min_y", "x_min"),
                 ("delta_y", "x_delta"), ("min_z", "z_min"), ("delta_z", "z_delta")):
        assert getattr(tr, a) == pytest.approx(float(g["h_" + b]), rel=1e-14, abs=0)
    for f in ("density", "density_x", "density_z", "vx", "vx_x"):
        ref = g["h_" + f]
        out = getattr(tr, f"data_{f}_interp")
        assert out.shape == ref.shape
        assert np.max(np.abs(out - ref)) <= 1e-11 * np.max(np.abs(ref)), f


@pytest.mark.parametrize("tag", ["dipole", "chicane_pos", "chicane_neg", "dipole_big"])
def test_wake_points(tag):
    g = golden(f"wake_{tag}.npz")
    run = oracle_from_wake_fixture(g)
    tr = run.tracker
    assert tr.data_density_interp.shape == g["h_density"].shape
    np.testing.assert_allclose(tr.data_density_interp, g["h_density"], rtol=0,
                               atol=1e-11 * np.max(np.abs(g["h_density"])))
    st = run.stats()
    assert st["slope"][0] == pytest.approx(float(g["slope"][0]), rel=1e-13)
    xm, zm, zr, xr = O.csr_mesh(st, *[int(v) if i < 2 else float(v)
                                      for i, v in enumerate(g["mesh_params"])])
    np.testing.assert_allclose(xm, g["xmesh"], rtol=1e-13, atol=1e-18)
    np.testing.assert_allclose(zm, g["zmesh"], rtol=1e-13, atol=1e-18)
    w = run.wake_oracle()
    for k, i in enumerate(g["points"]):
        dE, xk = w.wake(run.position + zm[i], xm[i])
        assert rel_err([dE], [g["wake_dE"][k]]) < 1e-9
        assert rel_err([xk], [g["wake_xkick"][k]]) < 1e-9
    if "mesh_dE" in g.files:
        dE, xk = w.points(run.position + zm, xm, nthreads=4)
        assert rel_err(dE, g["mesh_dE"].ravel()) < 1e-9
        assert rel_err(xk, g["mesh_xkick"].ravel()) < 1e-9


def test_wake_bitwise_on_reference_history():
    """Fed the reference's own history arrays and beam statistics, the C wake
    reproduces get_CSR_wake to the last bit (same IEEE operation order)."""
    from types import SimpleNamespace
    g = golden("wake_dipole.npz")
    tr = SimpleNamespace(
        data_density_interp=g["h_density"], data_density_x_interp=g["h_density_x"],
        data_density_z_interp=g["h_density_z"], data_vx_interp=g["h_vx"],
        data_vx_x_interp=g["h_vx_x"], min_x=float(g["h_t_min"]), min_y=float(g["h_x_min"]),
        min_z=float(g["h_z_min"]), delta_x=float(g["h_t_delta"]),
        delta_y=float(g["h_x_delta"]), delta_z=float(g["h_z_delta"]))
    from tests.helpers import lattice_from, integ_from
    lat = lattice_from(g)
    s, rho, dist, nsep, coords, nv, tau = O.reference_trajectory(lat, 2000)
    integ = integ_from(g)
    w = O.WakeOracle(tr, (s, rho, dist, coords, nv, tau), float(g["position"]),
                     float(g["sigma_z"]), float(g["sigma_x"]), float(g["slope"][0]),
                     float(g["mean_x"]), float(g["formation_length"]),
                     integ["n_formation_length"], integ["zbins"], integ["xbins"])
    for k, i in enumerate(g["points"]):
        dE, xk = w.wake(float(g["position"]) + g["zmesh"][i], g["xmesh"][i])
        assert dE == g["wake_dE"][k]
        assert xk == g["wake_xkick"][k]
    # debug integrands of the first point, region by region
    i = g["points"][0]
    dE, xk, buf = w.wake(float(g["position"]) + g["zmesh"][i], g["xmesh"][i], debug=True)
    nb = int(g["debug_n"])
    dbg = [g[f"debug_{j}"] for j in range(nb)]
    # unchirped layout: xp_w, xp_n, sp1, sp2, sp3, Iz1, Ix1, Iz2, Ix2, Iz3, Ix3
    xp_w, xp_n, sps, I = dbg[0], dbg[1], dbg[2:5], dbg[5:]
    off = 0
    for r in range(3):
        xp = xp_w if r == 0 else xp_n
        nxp, nsp = xp.size, sps[r].size
        np.testing.assert_array_equal(buf[off:off + nxp], xp); off += nxp
        np.testing.assert_array_equal(buf[off:off + nsp], sps[r]); off += nsp
        np.testing.assert_array_equal(buf[off:off + nxp * nsp].reshape(nxp, nsp), I[2 * r]); off += nxp * nsp
        np.testing.assert_array_equal(buf[off:off + nxp * nsp].reshape(nxp, nsp), I[2 * r + 1]); off += nxp * nsp


def test_step_plan_positions():
    from pydfcsr_gb300.synthetic import chicane_lattice
    p = StepPlan(chicane_lattice(0.065))
    assert len(p.positions) == 101
    assert p.positions[-1] == pytest.approx(6.5)


def test_apply_wakes_golden():
    """Beam.apply_wakes: pz (and px with the transverse kick) from the
    reference on a chirped beam, particles inside and outside the mesh."""
    g = golden("apply_wakes.npz")
    args = (g["dE_dct"], g["x_kick"], g["xrange"], g["zrange"], float(g["step_size"]),
            float(g["init_energy"]))
    for tag, transverse in (("t", True), ("l", False)):
        out = O.apply_wakes(g["coords"], *args, transverse, g["slope"])
        np.testing.assert_array_equal(out, g[f"out_{tag}"])
    moved = g["out_t"][5] != g["coords"][5]
    assert 0 < moved.sum() < moved.size      # some particles lie outside the mesh
