"""Reference-orbit tables of the lattice (host FP64, once per run) and their
device copies for the wake kernels.

``get_referece_traj`` keeps the reference's name and sampling
(pyDFCSR_2D/lattice.py:4-110): ``Nsample`` equispaced s points over the whole
lattice; in a dipole the orbit advances along a circle of radius L / angle, in
any other element along a straight line; n = (sin th, -cos th) and
tau = (cos th, sin th) with th the accumulated bend angle.  The recursion
(each sample built from the previous one) is kept as is: the wake reproduces
the reference's linear interpolation of these exact tables.
"""
from collections import OrderedDict

import numpy as np
import torch

__all__ = ["get_referece_traj", "Lattice"]


def get_referece_traj(lattice_config, Nsample=5000, Ndim=2):
    """Return s, rho, distance, nsep, coords, n_vec, tau_vec for a lattice
    dict whose first key is ``step_size`` and whose other keys are elements
    with ``type``, ``L`` (and ``angle`` for dipoles) and ``nsep``."""
    names = list(lattice_config.keys())[1:]
    n_el = len(names)
    distance = np.zeros(n_el)
    rho = np.zeros(n_el)
    nsep = np.zeros(n_el)
    total = 0.0
    for k, name in enumerate(names):
        el = lattice_config[name]
        nsep[k] = el["nsep"]
        if el["type"] == "dipole":
            rho[k] = el["angle"] / el["L"]
        total = el["L"] if k == 0 else el["L"] + total
        distance[k] = total
    s = np.linspace(0, distance[-1], Nsample)
    coords = np.zeros((Nsample, Ndim))
    tau_vec = np.zeros((Nsample, Ndim))
    n_vec = np.zeros((Nsample, Ndim))
    theta = 0
    tau_vec[0, 0], tau_vec[0, 1] = np.cos(theta), np.sin(theta)
    n_vec[0, 0], n_vec[0, 1] = np.sin(theta), -1 * np.cos(theta)
    el_idx = 0
    for k in range(1, Nsample):
        if s[k] > distance[el_idx]:
            el_idx += 1
        ds = s[k] - s[k - 1]
        el = lattice_config[names[el_idx]]
        if el["type"] == "dipole":
            L, angle = el["L"], el["angle"]
            phi = ds / L * angle
            radius = L / angle
            cx = coords[k - 1, 0] - radius * np.sin(theta)
            cy = coords[k - 1, 1] + radius * np.cos(theta)
            coords[k, 0] = cx + radius * np.sin(phi + theta)
            coords[k, 1] = cy - radius * np.cos(phi + theta)
        else:
            phi = 0
            coords[k, 0] = coords[k - 1, 0] + ds * np.cos(theta)
            coords[k, 1] = coords[k - 1, 1] + ds * np.sin(theta)
        theta += phi
        tau_vec[k, 0], tau_vec[k, 1] = np.cos(theta), np.sin(theta)
        n_vec[k, 0], n_vec[k, 1] = np.sin(theta), -1 * np.cos(theta)
    return s, rho, distance, nsep, coords, n_vec, tau_vec


class Lattice:
    """Lattice tables (pyDFCSR_2D/lattice.py:112-204) built from a dict.

    ``input_lattice`` is either the lattice dict itself (``step_size`` first,
    then elements) or ``{'lattice_input_file': path}`` (needs PyYAML).
    """

    def __init__(self, input_lattice, Nsample=2000):
        if "lattice_input_file" in input_lattice:
            lattice_config = _read_yaml(input_lattice["lattice_input_file"])
        else:
            lattice_config = input_lattice
        assert "step_size" in lattice_config, \
            "Required input parameter step_size to Lattice.__init__(**kwargs) was not found."
        self.lattice_config = lattice_config
        self._Nelement = len(lattice_config) - 1
        (self.s, self.rho, self.distance, self.nsep, self.coords, self.n_vec,
         self.tau_vec) = get_referece_traj(lattice_config, Nsample=Nsample)
        self._lattice_length = self.distance[-1]
        self.min_x, self.max_x = self.s[0], self.s[-1]
        self.delta_x = (self.max_x - self.min_x) / (self.s.shape[0] - 1)
        self.get_steps()
        self.current_element = None
        self._dev = None

    def get_steps(self):
        self.step_size = self.lattice_config["step_size"]
        self._positions_record = np.arange(0, self.lattice_length + self.step_size / 2, self.step_size)
        self._total_steps = len(self._positions_record)
        self.steps_per_element = np.zeros((self.Nelement,), dtype=int)
        prev = 0
        for k, d in enumerate(self.distance):
            ind = np.searchsorted(self._positions_record, d, side="right")
            self.steps_per_element[k] = ind - prev - 1 if k == 0 else ind - prev
            prev = ind

    @property
    def lattice_length(self):
        return self._lattice_length

    @property
    def total_steps(self):
        return self._total_steps

    @property
    def steps_record(self):
        return self._positions_record

    @property
    def Nelement(self):
        return self._Nelement

    def update(self, ele_name):
        self.current_element = ele_name

    def device_tables(self):
        """(table [Nsample, 6] = X0, Y0, nX, nY, tauX, tauY; rho; distance) as
        float64 CUDA tensors, cached."""
        if self._dev is None:
            tab = np.ascontiguousarray(np.concatenate([self.coords, self.n_vec, self.tau_vec], axis=1))
            dev = torch.device("cuda", torch.cuda.current_device())
            self._dev = (torch.from_numpy(tab).to(dev),
                         torch.from_numpy(np.ascontiguousarray(self.rho)).to(dev),
                         torch.from_numpy(np.ascontiguousarray(self.distance)).to(dev))
        return self._dev

    def device_deltas(self):
        """[Nsample, 6] float64 CUDA tensor of row differences of the table
        (row k+1 - row k, last row 0), cached: lets a linear interpolation be
        one fused multiply-add per table column."""
        if getattr(self, "_dev_delta", None) is None:
            tab = np.concatenate([self.coords, self.n_vec, self.tau_vec], axis=1)
            d = np.zeros_like(tab)
            d[:-1] = tab[1:] - tab[:-1]
            dev = torch.device("cuda", torch.cuda.current_device())
            self._dev_delta = torch.from_numpy(np.ascontiguousarray(d)).to(dev)
        return self._dev_delta

    def device_tables_dw(self):
        """(table, row differences) as [Nsample, 6, 2] float32 CUDA tensors of
        double-word pairs (hi, lo), cached: the mixed wake's geometry runs in
        double-word FP32 from these."""
        if getattr(self, "_dev_dw", None) is None:
            tab = np.concatenate([self.coords, self.n_vec, self.tau_vec], axis=1)
            d = np.zeros_like(tab)
            d[:-1] = tab[1:] - tab[:-1]
            dev = torch.device("cuda", torch.cuda.current_device())
            self._dev_dw = (torch.from_numpy(_double_word(tab)).to(dev),
                            torch.from_numpy(_double_word(d)).to(dev))
        return self._dev_dw


def _double_word(a):
    """float32 pairs (hi, lo) with hi + lo the float64 value to ~48 bits."""
    hi = a.astype(np.float32)
    lo = (a - hi.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(np.stack([hi, lo], axis=-1))


def _read_yaml(path):
    try:
        import yaml
    except ImportError as e:  # pragma: no cover - PyYAML is optional
        raise ImportError("reading a lattice file needs PyYAML; pass the lattice dict instead") from e
    class _Loader(yaml.SafeLoader):
        pass
    _Loader.add_constructor(yaml.resolver.BaseResolver.DEFAULT_MAPPING_TAG,
                            lambda loader, node: OrderedDict(loader.construct_pairs(node)))
    with open(path) as f:
        return yaml.load(f, _Loader)
