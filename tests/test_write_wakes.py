"""CSR2D.write_wakes: the HDF5 layout of CSR.py:799-835, checked on the CPU.

h5py is not installed here, so a small stand-in module records what would be
written (groups, attributes, datasets) into the file as a pickle; the test
reads that back and checks group names, attributes, dataset names, shapes
and values against the layout the reference writes.
"""
import os
import pickle
import sys
import types

import numpy as np
import pytest

from pydfcsr_gb300.CSR import CSR2D
from pydfcsr_gb300.params import CSR_params


class _Node(dict):
    def __init__(self):
        super().__init__()
        self.attrs = {}

    def create_group(self, name):
        assert name not in self, f"group {name} exists"
        self[name] = _Node()
        return self[name]

    def create_dataset(self, name, data):
        assert name not in self
        self[name] = np.array(data, copy=True)
        return self[name]


class _File(_Node):
    def __init__(self, name, mode):
        super().__init__()
        assert mode == "a"
        self._name = name
        if os.path.isfile(name):
            with open(name, "rb") as f:
                self.update(pickle.load(f))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        with open(self._name, "wb") as f:
            pickle.dump(dict(self), f)


@pytest.fixture
def fake_h5py(monkeypatch):
    mod = types.ModuleType("h5py")
    mod.File = _File
    monkeypatch.setitem(sys.modules, "h5py", mod)


def _csr(tmp_path, step, xbins=4, zbins=6):
    csr = object.__new__(CSR2D)
    csr.CSR_params = CSR_params({"workdir": str(tmp_path), "write_name": "chicane",
                                 "xbins": xbins, "zbins": zbins})
    csr.timestamp = "2026-01-01T00_00_00+00_00"
    csr.beam = types.SimpleNamespace(step=step, position=0.25 * step, init_gamma=1956.95,
                                     init_energy=1e9, charge=1e-9)
    csr.lattice = types.SimpleNamespace(current_element="B1")
    csr._pending = None
    csr._mesh = (-3e-5, 3e-5, xbins, -1e-4, 1e-4, zbins, 0.5, 1e-6, csr.beam.position)
    csr._mesh_host = None
    rng = np.random.default_rng(step)
    csr.dE_dct = rng.standard_normal((xbins, zbins))
    csr.x_kick = rng.standard_normal((xbins, zbins))
    return csr


def test_write_wakes_layout(tmp_path, fake_h5py):
    written = {}
    for step in (1, 2):
        csr = _csr(tmp_path, step)
        fn = csr.write_wakes()
        written[step] = (csr.dE_dct, csr.x_kick, csr.CSR_xmesh, csr.CSR_zmesh)
    assert fn == os.path.join(str(tmp_path), "chicane-2026-01-01T00_00_00+00_00-wakes.h5")
    with open(fn, "rb") as f:
        root = pickle.load(f)
    assert sorted(root) == ["step_1", "step_2"]
    for step, (dE, xk, xm, zm) in written.items():
        g = root[f"step_{step}"]
        assert g.attrs == {"step": step, "position": 0.25 * step, "mean_gamma": 1956.95,
                           "beam_energy": 1e9, "element": "B1", "charge": 1e-9}
        assert sorted(g) == ["longitudinal", "transverse"]
        lon, tra = g["longitudinal"], g["transverse"]
        assert lon.attrs == {"unit": "MeV/m"} and tra.attrs == {"unit": "MeV/m"}
        assert sorted(lon) == ["dE_dct", "x_grids", "z_grids"]
        assert sorted(tra) == ["x_grids", "xkicks", "z_grids"]
        for sub in (lon, tra):
            assert sub["x_grids"].shape == (4, 6) and np.array_equal(sub["x_grids"].ravel(), xm)
            assert np.array_equal(sub["z_grids"].ravel(), zm)
        assert np.array_equal(lon["dE_dct"], dE) and np.array_equal(tra["xkicks"], xk)
    # the mesh in the file is the reference's: x slow, z fast, chirp added back
    z = np.linspace(-1e-4, 1e-4, 6)
    x = np.linspace(-3e-5, 3e-5, 4)
    assert np.array_equal(root["step_1"]["longitudinal"]["z_grids"], np.tile(z, (4, 1)))
    assert np.array_equal(root["step_1"]["longitudinal"]["x_grids"],
                          x[:, None] + np.polyval([0.5, 1e-6], z)[None, :])


def test_write_wakes_step1_replaces_file(tmp_path, fake_h5py):
    _csr(tmp_path, 1).write_wakes()
    _csr(tmp_path, 2).write_wakes()
    fn = _csr(tmp_path, 1).write_wakes()
    with open(fn, "rb") as f:
        assert sorted(pickle.load(f)) == ["step_1"]


def test_write_wakes_needs_h5py(tmp_path, monkeypatch):
    monkeypatch.setitem(sys.modules, "h5py", None)
    with pytest.raises(ImportError, match="h5py"):
        _csr(tmp_path, 1).write_wakes()


def test_prefix_and_timestamp_format():
    """<write_name>-<ISO time, ':' replaced by '_'> as the reference's
    isotime (tools.py:16-22) and CSR2D.prefix (CSR.py:41)."""
    import re
    from pydfcsr_gb300.CSR import _isotime
    ts = _isotime()
    assert ":" not in ts
    assert re.fullmatch(r"\d{4}-\d\d-\d\dT\d\d_\d\d_\d\d[+-]\d\d_\d\d", ts)
    csr = object.__new__(CSR2D)
    csr.CSR_params = CSR_params({"write_name": "run7"})
    csr.timestamp = ts
    assert csr.prefix == f"run7-{ts}"
