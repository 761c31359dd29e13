"""Generate the golden fixtures of the wake path by running the reference itself.

Run in a container that holds the pyDFCSR_2D source tree (read-only is fine),
giving the directory that contains ``pyDFCSR_2D/``; optional fixture names
after it regenerate only those fixtures:

    python tests/golden/make_golden.py <reference checkout> [r_gen6 ...]

The reference is imported through ``ref_shim`` (stub modules for numba,
bmadx, h5py, mpi4py, yaml, distgen, pmd_beamphysics and matplotlib; numba
loops run as plain Python with the same IEEE double arithmetic).  Every input
and every output is stored in the ``.npz`` files beside this script, so tests
never need the reference at run time.

Fixtures:
  interp.npz    interpolate3D known answer (scipy docs grid 11x22x33 and the
                notebook grid 200x200x100) plus random / edge queries;
                interpolate1D random / edge queries.
  cic.npz       histogram_cic_2d on hand-placed edge particles and on a seeded
                beam (w = 1 and w = px), non-square grid.
  df.npz        DF_tracker.get_DF for a round beam (fallback grid rule) and a
                chirped beam (configured grid rule).
  lattice.npz   get_referece_traj tables for a dipole and a chicane.
  history.npz   a multi-step get_DF / append_DF / append_interpolant /
                build_interpolant sequence with a re-interpolation event and
                window trimming (pop_left_DF).
  wake_*.npz    get_CSR_mesh, get_CSR_wake (with debug integrands) and
                calculate_2D_CSR for an unchirped dipole and for both signs of
                chirp (the 4-region branch).
  apply_wakes.npz  Beam.apply_wakes with and without the transverse kick.
  r_gen6.npz    r_gen6 matrices (drift, sector and rectangular bends with
                edges and half gap, quadrupoles of both signs, combined
                function, rolls, the pure rotation) and the three tracked
                vectors of the reference's BmadX tracking notebook.
"""
import os
import sys
import time
from collections import OrderedDict
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import ref_shim  # noqa: E402
from pydfcsr_gb300.synthetic import (gaussian_beam, dipole_lattice,  # noqa: E402
                                     chicane_lattice, StepPlan)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {name}: {os.path.getsize(path) / 1024:.1f} KiB")


def gen_interp(R):
    out = {}
    x = np.linspace(1, 4, 11); y = np.linspace(4, 7, 22); z = np.linspace(7, 9, 33)
    xg, yg, zg = np.meshgrid(x, y, z, indexing="ij")
    d = 2 * xg ** 3 + 3 * yg ** 2 - zg
    dx, dy, dz = np.mean(np.diff(x)), np.mean(np.diff(y)), np.mean(np.diff(z))
    q = np.array([[2.1, 6.2, 8.3], [3.3, 5.2, 7.1]])
    out["ka_small_data"] = d
    out["ka_small_q"] = q
    out["ka_small_delta"] = np.array([dx, dy, dz])
    out["ka_small_out"] = R.interp3D.interpolate3D(q[:, 0], q[:, 1], q[:, 2], d, 1., 4., 7., dx, dy, dz)

    x = np.linspace(1, 4, 200); y = np.linspace(4, 7, 200); z = np.linspace(7, 9, 100)
    xg, yg, zg = np.meshgrid(x, y, z, indexing="ij")
    d = 2 * xg ** 3 + 3 * yg ** 2 - zg
    dx, dy, dz = np.mean(np.diff(x)), np.mean(np.diff(y)), np.mean(np.diff(z))
    out["ka_big_delta"] = np.array([dx, dy, dz])
    out["ka_big_out"] = R.interp3D.interpolate3D(np.array([2.1]), np.array([6.2]), np.array([8.3]),
                                                 d, 1., 4., 7., dx, dy, dz)

    # Random + edge queries on a small random grid: covers the (-1, 0)
    # truncation band (linear extrapolation), the clamp on the last index,
    # and out-of-range zeros.
    rng = np.random.default_rng(11)
    data = rng.normal(size=(7, 9, 12))
    mins = np.array([0.5, -1.0, 2.0]); deltas = np.array([0.25, 0.1, 0.05])
    m = 4000
    u = rng.uniform(-1.6, 1.6, size=(3, m)) * np.array([[7], [9], [12]])
    u = np.where(rng.random((3, m)) < 0.5, np.abs(u), u)
    edges = np.array([[-1.0, -0.999, -0.5, 0.0, 5.999, 6.0, 6.5, 6.99, 7.0, 7.2],
                      [-1.0, -0.2, 0.0, 3.3, 7.999, 8.0, 8.5, 8.9999, 9.0, 10.],
                      [-1.0, -0.7, 0.0, 5.5, 10.99, 11.0, 11.5, 11.9, 12.0, 13.]])
    u = np.concatenate([u, edges], axis=1)
    qv = mins[:, None] + u * deltas[:, None]
    out["rnd_data"] = data
    out["rnd_min"] = mins
    out["rnd_delta"] = deltas
    out["rnd_q"] = qv
    out["rnd_out"] = R.interp3D.interpolate3D(qv[0], qv[1], qv[2], data, *mins, *deltas)

    tab = rng.normal(size=50)
    u1 = np.concatenate([rng.uniform(-3, 53, 3000),
                         [-1.0, -0.99, -0.3, 0.0, 48.9, 49.0, 49.5, 49.999, 50.0, 51.0]])
    q1 = -2.0 + u1 * 0.125
    out["i1_tab"] = tab
    out["i1_q"] = q1
    out["i1_out"] = R.interp1D.interpolate1D(q1, tab, -2.0, 0.125)
    save("interp.npz", **out)


def gen_cic(R):
    out = {}
    nb1, lo1, hi1 = 6, -1.0, 2.0
    nb2, lo2, hi2 = 5, 0.0, 1.0
    sp1 = (hi1 - lo1) / nb1; sp2 = (hi2 - lo2) / nb2
    q1 = [lo1, lo1 + sp1, hi1, hi1 - 1e-12, lo1 - 0.3 * sp1, lo1 - sp1, lo1 - 1.2 * sp1,
          hi1 + 0.2 * sp1, 0.3, 0.31, 0.9, 1.1, -0.7, 1.7]
    q2 = [lo2, hi2, lo2 + 2 * sp2, 0.5, 0.55, lo2 - 0.5 * sp2, 0.1, 0.95, hi2 + 0.1 * sp2,
          lo2 - 1.0 * sp2, 0.33, 0.77, 0.21, 0.99]
    q1 = np.array(q1, dtype=float); q2 = np.array(q2, dtype=float)
    w = np.linspace(0.5, 2.0, q1.size)
    out["edge_q1"], out["edge_q2"], out["edge_w"] = q1, q2, w
    out["edge_grid"] = np.array([nb1, lo1, hi1, nb2, lo2, hi2])
    out["edge_out"] = R.deposit.histogram_cic_2d(q1, q2, w, nb1, lo1, hi1, nb2, lo2, hi2)

    b = gaussian_beam(8000, 10e-6, 20e-6, 1e-4, 5e-6, 0.0, seed=7)
    x, px, z = b[0], b[1], b[4]
    g = (48, x.mean() - 4 * x.std(), x.mean() + 4 * x.std(), 64, z.mean() - 4.5 * z.std(),
         z.mean() + 4.5 * z.std())
    out["beam_x"], out["beam_z"], out["beam_px"] = x, z, px
    out["beam_grid"] = np.array(g, dtype=float)
    out["beam_out_ones"] = R.deposit.histogram_cic_2d(x, z, np.ones(x.shape), *g)
    out["beam_out_px"] = R.deposit.histogram_cic_2d(x, z, px, *g)
    save("cic.npz", **out)


def df_case(R, beam, params):
    t = R.deposit.DF_tracker(params)
    t.get_DF(x=beam[0], z=beam[4], px=beam[1], t=0.25)
    return {k: getattr(t, k) for k in ("x_grids", "z_grids", "density", "vx",
                                       "density_x", "density_z", "vx_x")}


def gen_df(R):
    out = {}
    p = {"xbins": 64, "zbins": 80, "xlim": 5, "zlim": 5, "filter_order": 2,
         "filter_window": 9, "velocity_threhold": 1000}
    # Round beam: sigma_x / sigma_x(slice) ~ 1 -> reference falls back to
    # 100x100 with window 5 (pyDFCSR_2D/deposit.py:157-168).
    b = gaussian_beam(10000, 10e-6, 20e-6, 1e-4, 5e-6, 0.0, seed=21)
    for k, v in df_case(R, b, p).items():
        out["round_" + k] = v
    out["round_x"], out["round_z"], out["round_px"] = b[0], b[4], b[1]
    # Strongly x-z correlated beam: frac > 5 -> configured grid and window.
    b = gaussian_beam(10000, 2e-6, 20e-6, 1e-4, 5e-6, 0.0, seed=22)
    b[0] += 2.0 * b[4]
    b[1] += 3e-2 * b[4]
    for k, v in df_case(R, b, p).items():
        out["tilt_" + k] = v
    out["tilt_x"], out["tilt_z"], out["tilt_px"] = b[0], b[4], b[1]
    p1 = dict(p, filter_order=1, velocity_threhold=5)
    for k, v in df_case(R, b, p1).items():
        out["tilt1_" + k] = v
    out["params"] = np.array([64, 80, 5, 5, 2, 9, 1000], dtype=float)
    save("df.npz", **out)


def gen_lattice(R):
    out = {}
    for tag, lat in (("dipole", dipole_lattice(1.5, 0.3, 0.001)),
                     ("chicane", chicane_lattice(0.065))):
        s, rho, dist, nsep, coords, n_vec, tau_vec = R.lattice.get_referece_traj(lat, Nsample=2000)
        out[tag + "_s"], out[tag + "_rho"], out[tag + "_distance"] = s, rho, dist
        out[tag + "_coords"], out[tag + "_n_vec"], out[tag + "_tau_vec"] = coords, n_vec, tau_vec
        elems = list(lat.keys())[1:]
        out[tag + "_elements"] = np.array(
            [[lat[e]["L"], lat[e].get("angle", 0.0), 1.0 if lat[e]["type"] == "dipole" else 0.0]
             for e in elems])
    save("lattice.npz", **out)


class RefRun:
    """Drive the reference's DF / history / wake methods over synthetic steps.

    Mirrors the call order of ``CSR2D.initialization`` and ``CSR2D.run``
    (``pyDFCSR_2D/CSR.py:75-78, 297-329``) with r_gen6 transport in place of
    bmadx tracking.
    """

    def __init__(self, R, lattice, beam, dep, integ, mesh, charge=1e-9):
        self.R = R
        self.plan = StepPlan(lattice)
        self.beam6 = beam.copy()
        csr = object.__new__(R.CSR.CSR2D)
        csr.DF_tracker = R.deposit.DF_tracker(dep)
        csr.integration_params = SimpleNamespace(**integ)
        csr.CSR_params = SimpleNamespace(**mesh)
        lat = SimpleNamespace()
        (lat.s, lat.rho, lat.distance, lat.nsep, lat.coords, lat.n_vec,
         lat.tau_vec) = R.lattice.get_referece_traj(lattice, Nsample=2000)
        lat.min_x, lat.max_x = lat.s[0], lat.s[-1]
        lat.delta_x = (lat.max_x - lat.min_x) / (lat.s.shape[0] - 1)
        lat.Nelement = len(lattice) - 1
        csr.lattice = lat
        csr.CSR_scaling = 8.98755e3 * charge
        csr.parallel = False
        self.csr = csr
        self.position = 0.0
        self.update_beam()

    def update_beam(self):
        b = self.beam6
        x, z = b[0], b[4]
        slope = np.polyfit(z, x, deg=1)
        self.csr.beam = SimpleNamespace(
            position=self.position, x=x, z=z, px=b[1],
            _sigma_x=np.std(x), _sigma_z=np.std(z), _slope=slope,
            _mean_x=np.mean(x), _mean_z=np.mean(z),
            sigma_x=np.std(x), sigma_z=np.std(z), slope=slope,
            mean_x=np.mean(x), mean_z=np.mean(z),
            x_transform=x - np.polyval(slope, z))

    def df_step(self, formation_length):
        c = self.csr
        c.DF_tracker.get_DF(x=c.beam.x, z=c.beam.z, px=c.beam.px, t=c.beam.position)
        c.DF_tracker.append_DF()
        c.DF_tracker.append_interpolant(formation_length=formation_length,
                                        n_formation_length=c.integration_params.n_formation_length)

    def init(self):
        self.df_step(float("inf"))

    def step(self, k):
        self.beam6 = self.plan.matrix(k) @ self.beam6
        self.position = self.plan.positions[k]
        self.update_beam()
        lf = self.plan.formation_length(k, self.csr.beam.sigma_z)
        self.csr.formation_length = lf
        self.df_step(lf)
        self.csr.DF_tracker.build_interpolant()
        return lf


def history_arrays(tr):
    return {
        "t_min": tr.min_x, "x_min": tr.min_y, "z_min": tr.min_z,
        "t_delta": tr.delta_x, "x_delta": tr.delta_y, "z_delta": tr.delta_z,
        "time_interp": np.array(tr.time_interp),
        "x_grid_interp": tr.x_grid_interp, "z_grid_interp": tr.z_grid_interp,
        "density": tr.data_density_interp, "density_x": tr.data_density_x_interp,
        "density_z": tr.data_density_z_interp, "vx": tr.data_vx_interp,
        "vx_x": tr.data_vx_x_interp,
    }


def gen_history(R):
    """Beam whose sigma_x grows 2.5x over the steps: forces a re-interpolation
    of all slices; a short formation length trims the window."""
    lat = OrderedDict(step_size=0.01)
    lat["D1"] = {"type": "drift", "L": 0.08, "nsep": 1}
    beam = gaussian_beam(6000, 10e-6, 20e-6, 1e-4, 3e-4, 0.0, seed=31)
    dep = {"xbins": 40, "zbins": 48, "xlim": 5, "zlim": 5, "filter_order": 2,
           "filter_window": 5, "velocity_threhold": 1000, "upper_limit": 30}
    run = RefRun(R, lat, beam, dep, {"n_formation_length": 1.0, "zbins": 10, "xbins": 10},
                 {"xbins": 4, "zbins": 4, "xlim": 3, "zlim": 3})
    out = {"beam0": beam.copy(), "positions": run.plan.positions}
    run.init()
    lfs = []
    steps_out = []
    for k in range(1, len(run.plan.positions)):
        # override the drift's accumulated formation length with a short window
        run.beam6 = run.plan.matrix(k) @ run.beam6
        run.position = run.plan.positions[k]
        run.update_beam()
        lf = 0.025
        run.csr.formation_length = lf
        run.df_step(lf)
        run.csr.DF_tracker.build_interpolant()
        lfs.append(lf)
        steps_out.append(len(run.csr.DF_tracker.time_interp))
    out["formation_lengths"] = np.array(lfs)
    out["n_slices"] = np.array(steps_out)
    out["sigma_x_interp"] = run.csr.DF_tracker.sigma_x_interp
    out["sigma_z_interp"] = run.csr.DF_tracker.sigma_z_interp
    for k, v in history_arrays(run.csr.DF_tracker).items():
        out["h_" + k] = v
    out["dep"] = np.array([40, 48, 5, 5, 2, 5, 1000, 30], dtype=float)
    save("history.npz", **out)


def gen_wake(R, tag, lattice, beam, n_steps, dep, integ, mesh, points, debug_point=0,
             full_mesh=True):
    run = RefRun(R, lattice, beam, dep, integ, mesh)
    out = {"beam0": beam.copy(), "positions": run.plan.positions[: n_steps + 1]}
    out["lattice_step"] = lattice["step_size"]
    out["lattice_elements"] = np.array(
        [[lattice[e]["L"], lattice[e].get("angle", 0.0), 1.0 if lattice[e]["type"] == "dipole" else 0.0]
         for e in list(lattice.keys())[1:]])
    run.init()
    lf = None
    for k in range(1, n_steps + 1):
        lf = run.step(k)
    c = run.csr
    c.get_CSR_mesh()
    out["formation_length"] = lf
    out["position"] = c.beam.position
    out["slope"] = c.beam._slope
    out["sigma_x"], out["sigma_z"] = c.beam._sigma_x, c.beam._sigma_z
    out["mean_x"], out["mean_z"] = c.beam._mean_x, c.beam._mean_z
    out["xmesh"], out["zmesh"] = c.CSR_xmesh, c.CSR_zmesh
    out["zrange"], out["xrange"] = c.CSR_zrange, c.CSR_xrange_transformed
    for k, v in history_arrays(c.DF_tracker).items():
        out["h_" + k] = v
    wz, wx = [], []
    t0 = time.time()
    for i in points:
        s = c.beam.position + c.CSR_zmesh[i]
        a, b = c.get_CSR_wake(s, c.CSR_xmesh[i])
        wz.append(a); wx.append(b)
    out["points"] = np.array(points)
    out["wake_dE"], out["wake_xkick"] = np.array(wz), np.array(wx)
    i = points[debug_point]
    dbg = c.get_CSR_wake(c.beam.position + c.CSR_zmesh[i], c.CSR_xmesh[i], debug=True)
    out["debug_n"] = len(dbg)
    for j, arr in enumerate(dbg):
        out[f"debug_{j}"] = arr
    if full_mesh:
        c.calculate_2D_CSR()
        out["mesh_dE"], out["mesh_xkick"] = c.dE_dct, c.x_kick
    out["integ"] = np.array([integ["n_formation_length"], integ["zbins"], integ["xbins"]])
    out["mesh_params"] = np.array([mesh["xbins"], mesh["zbins"], mesh["xlim"], mesh["zlim"]])
    out["dep"] = np.array([dep["xbins"], dep["zbins"], dep["xlim"], dep["zlim"],
                           dep["filter_order"], dep["filter_window"], dep["velocity_threhold"],
                           dep.get("upper_limit", -1)], dtype=float)
    print(f"  {tag}: {len(points)} wake points in {time.time() - t0:.1f}s; slope={c.beam._slope[0]:.3g}")
    save(f"wake_{tag}.npz", **out)


def gen_apply_wakes(R):
    """Beam.apply_wakes (beams.py:108-131) on a chirped beam: a wake table on
    a 9 x 11 mesh (CSR_xrange_transformed x CSR_zrange), particles inside and
    outside the mesh, with and without the transverse kick."""
    import collections
    import pyDFCSR_2D.beams as B
    Part = collections.namedtuple("Particle", "x px y py z pz s p0c mc2")
    B.Particle = Part          # the shim's bmadx stand-in carries no fields
    coords = gaussian_beam(1500, 20e-6, 50e-6, 1e-4, 5e-6, -10.0, seed=44)
    coords[0] += 1.1 * coords[4]          # x-z correlation: x_transform != x
    rng = np.random.default_rng(45)
    x, z = coords[0], coords[4]
    p = np.polyfit(z, x, deg=1)
    xt = x - np.polyval(p, z)
    xr = np.linspace(xt.mean() - 2.5 * xt.std(), xt.mean() + 2.5 * xt.std(), 9)
    zr = np.linspace(z.mean() - 2.5 * z.std(), z.mean() + 2.5 * z.std(), 11)
    dE = rng.normal(0.0, 2.0, (9, 11))
    xk = rng.normal(0.0, 0.5, (9, 11))
    out = {"coords": coords, "xrange": xr, "zrange": zr, "dE_dct": dE, "x_kick": xk,
           "step_size": np.array(0.013), "init_energy": np.array(1e9), "slope": p}
    for tag, transverse in (("t", True), ("l", False)):
        b = object.__new__(B.Beam)
        b.particle = Part(*[coords[k].copy() for k in range(6)], 0.0, 1e9, 0.511e6)
        b._init_energy = 1e9
        b.apply_wakes(dE, xk, xr, zr, 0.013, transverse)
        out[f"out_{tag}"] = np.array([getattr(b.particle, f) for f in ("x", "px", "y", "py", "z", "pz")])
    save("apply_wakes.npz", **out)


def gen_interfaces(R):
    """interfaces.py:13-127 on a small beam: openPMD -> bmadx coordinates,
    and bmadx -> openPMD data from numpy and from torch particles.  The
    shim's bmadx Particle and ParticleGroup are replaced by a namedtuple and
    a function returning the data dict, so the reference's arithmetic is
    recorded as is."""
    import collections
    import types
    import torch
    import pyDFCSR_2D.interfaces as I
    Part = collections.namedtuple("Particle", "x px y py z pz s p0c mc2")
    I.Particle = Part
    I.ParticleGroup = lambda data: data
    rng = np.random.default_rng(46)
    n, p0c = 128, 1.0e9
    pmd = types.SimpleNamespace(x=rng.normal(0, 2e-5, n), px=rng.normal(0, 5e3, n),
                                y=rng.normal(0, 1e-5, n), py=rng.normal(0, 3e3, n),
                                z=rng.normal(0, 5e-5, n), p=p0c * (1 + rng.normal(0, 1e-3, n)))
    coords = np.array(I.openpmd_to_bmadx_coords(pmd, p0c))
    part = I.openpmd_to_bmadx_particles(pmd, p0c, s=0.37)
    out = {"x": pmd.x, "px": pmd.px, "y": pmd.y, "py": pmd.py, "z": pmd.z, "p": pmd.p,
           "p0c": np.array(p0c), "s": np.array(0.37), "charge": np.array(1e-9),
           "coords": coords, "mc2": np.array(part.mc2)}
    keys = ("x", "px", "y", "py", "z", "pz", "t", "weight")
    dat = I.bmadx_particles_to_openpmd(part, 1e-9)
    out["pmd_numpy"] = np.array([dat[k] for k in keys])
    tpart = Part(*[torch.from_numpy(c.copy()) for c in coords], 0.37, p0c, part.mc2)
    dat = I.bmadx_particles_to_openpmd(tpart, 1e-9)
    out["pmd_torch"] = np.array([dat[k] for k in keys])
    save("interfaces.npz", **out)


R_GEN6_CASES = [
    # (L, angle, k1, roll, E1, E2, hgap)
    (1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0),           # drift (notebook)
    (0.1, 0.05, 0.0, 0.0, 0.0, 0.1, 0.0),          # sbend with exit edge (notebook)
    (0.1, 0.0, 10.0, 0.0, 0.0, 0.0, 0.0),          # focusing quad (notebook)
    (0.2, 0.0, -7.5, 0.0, 0.0, 0.0, 0.0),          # defocusing quad
    (0.5, 0.05, 0.0, 0.0, 0.0, 0.0, 0.0),          # chicane sector bend
    (0.5, -0.05, 0.0, 0.0, 0.0, 0.0, 0.0),
    (0.3, 0.2, 0.0, 0.0, 0.1, 0.1, 0.0),           # rectangular bend
    (0.3, 0.2, 0.0, 0.0, 0.1, 0.1, 0.02),          # with fringe-field half gap
    (0.4, 0.1, 1.5, 0.0, 0.0, 0.0, 0.0),           # combined function
    (0.4, 0.1, -3.0, 0.3, 0.02, -0.03, 0.01),      # rolled combined function, edges
    (0.2, 0.0, 5.0, np.pi / 4, 0.0, 0.0, 0.0),     # skew quad
    (0.0, 0.0, 0.0, 0.7, 0.0, 0.0, 0.0),           # pure rotation
    (0.25, 1e-13, 0.0, 0.0, 0.0, 0.0, 0.0),        # almost no bend
]


def gen_r_gen6(R):
    """r_gen6 (r_gen6.py:4-122) on the cases above, and R @ (1e-3 * ones(6))
    for the notebook's three elements (test/test_BmadX_tracking.ipynb)."""
    cases = np.array(R_GEN6_CASES, dtype=np.float64)
    mats = np.array([R.r_gen6.r_gen6(L=c[0], angle=c[1], k1=c[2], roll=c[3], E1=c[4], E2=c[5],
                                     hgap=c[6]) for c in cases])
    coords = np.ones(6) * 1e-3
    tracked = np.array([np.matmul(mats[k], coords) for k in range(3)])
    save("r_gen6.npz", cases=cases, mats=mats, tracked=tracked)


def gen_wakes(R):
    dep = {"xbins": 40, "zbins": 48, "xlim": 5, "zlim": 5, "filter_order": 2,
           "filter_window": 5, "velocity_threhold": 1000, "upper_limit": 36}
    integ = {"n_formation_length": 1.5, "zbins": 16, "xbins": 12}
    mesh = {"xbins": 4, "zbins": 5, "xlim": 3, "zlim": 3}
    # Unchirped dipole (3-region branch): rho = 1.5 m, 20 mm steps.
    lat = dipole_lattice(1.5, 0.3, 0.02)
    beam = gaussian_beam(6000, 10e-6, 20e-6, 1e-4, 5e-6, 0.0, seed=41)
    gen_wake(R, "dipole", lat, beam, 12, dep, integ, mesh, points=[0, 7, 10, 12, 19])
    # Chicane with chirp: |slope| > 1 late in the first long drift -> the
    # 4-region branch; chirp +10 / -10 1/m gives both signs of slope.
    lat = chicane_lattice(0.13)
    beam = gaussian_beam(6000, 20e-6, 50e-6, 1e-4, 5e-6, 10.0, seed=42)
    gen_wake(R, "chicane_pos", lat, beam, 18, dep, integ, mesh, points=[0, 6, 9, 13, 19])
    beam = gaussian_beam(6000, 20e-6, 50e-6, 1e-4, 5e-6, -10.0, seed=43)
    gen_wake(R, "chicane_neg", lat, beam, 18, dep, integ, mesh, points=[1, 8, 11, 18],
             full_mesh=False)
    # One point at production integration size (100 x 100 bins).
    integ_big = {"n_formation_length": 1.5, "zbins": 100, "xbins": 100}
    lat = dipole_lattice(1.5, 0.3, 0.02)
    beam = gaussian_beam(6000, 10e-6, 20e-6, 1e-4, 5e-6, 0.0, seed=41)
    gen_wake(R, "dipole_big", lat, beam, 12, dep, integ_big, mesh, points=[12],
             full_mesh=False)


GENERATORS = {"interfaces": gen_interfaces, "apply_wakes": gen_apply_wakes, "interp": gen_interp,
              "cic": gen_cic, "df": gen_df, "lattice": gen_lattice, "history": gen_history,
              "wake": gen_wakes, "r_gen6": gen_r_gen6}


def main(ref_root, only=None):
    R = ref_shim.install(ref_root)
    want = list(only or GENERATORS)
    bad = [w for w in want if w not in GENERATORS]
    if bad:
        raise SystemExit(f"unknown fixtures {bad}; choose from {sorted(GENERATORS)}")
    for name in want:
        GENERATORS[name](R)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py <directory holding pyDFCSR_2D/> [fixture ...]")
    main(sys.argv[1], sys.argv[2:] or None)
