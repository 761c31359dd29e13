"""Step driver for synthetic workloads on the GPU.

Reproduces the call order of ``CSR2D.run`` (pyDFCSR_2D/CSR.py:202-358) for the
wake path - transport, get_DF, append_DF, append_interpolant,
build_interpolant, get_CSR_mesh, calculate_2D_CSR - with r_gen6 linear
transport in place of bmadx.  ``host_transport=True`` transports on the host
in FP64 numpy (bit-identical particles to a CPU run of the same plan);
otherwise the 6x6 matrices are applied on the device (dfcsr_transport6).
"""
import numpy as np

from .beams import Beam
from .CSR import CSR2D
from .synthetic import StepPlan

__all__ = ["WakeRun"]


class WakeRun:
    def __init__(self, lattice, beam6, deposit, integration, mesh, precision="fp64",
                 grid_rule="reference", charge=1e-9, energy=1e9, near_band=0.0,
                 host_transport=True):
        self.plan = StepPlan(lattice)
        self.host_transport = host_transport
        self.coords = np.array(beam6, dtype=np.float64, copy=True) if host_transport else None
        self.beam = Beam(beam6, charge=charge, energy=energy, position=0.0)
        self.csr = CSR2D(beam=self.beam, lattice=lattice, particle_deposition=deposit,
                         CSR_integration=integration, CSR_computation=mesh, precision=precision,
                         grid_rule=grid_rule, near_band=near_band)
        self.k = 0

    def step(self, k=None, coords=None):
        """Advance to step k (default: next) and update the history."""
        k = self.k + 1 if k is None else k
        if coords is not None:
            self.beam.set_coords(coords)
        elif self.host_transport:
            self.coords = self.plan.matrix(k) @ self.coords
            self.beam.set_coords(self.coords)
        else:
            self.beam.transport(self.plan.matrix(k))
            self.beam.update_status()
        self.beam.position = float(self.plan.positions[k])
        self.beam.step = k
        lf = self.plan.formation_length(k, self.beam.sigma_z)
        self.csr.update_history(lf)
        self.k = k
        return lf

    def wake(self, precision=None):
        """Mesh and wake at the current step; returns (dE_dct, x_kick) numpy."""
        self.csr.get_CSR_mesh()
        self.csr.calculate_2D_CSR(precision)
        return self.csr.dE_dct, self.csr.x_kick
