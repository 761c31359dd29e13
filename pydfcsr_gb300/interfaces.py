"""Particle format conversions: the call surface of ``pyDFCSR_2D.interfaces``.

The reference converts between openPMD-beamphysics ``ParticleGroup`` objects
and bmadx ``Particle`` coordinates (interfaces.py:13-127).  Neither
package is needed here:
- ``openpmd_to_bmadx_coords`` reads any object with ``x, px, y, py, z, p``
  arrays;
- ``openpmd_to_bmadx_particles`` returns a bmadx ``Particle`` when bmadx is
  installed, else this module's :class:`Particle` tuple with the same fields;
- ``bmadx_particles_to_openpmd`` returns a ``ParticleGroup`` when
  pmd_beamphysics is installed, else the data dict that would build one.

Particle arrays may be numpy or torch (interfaces.py:78-94).
:meth:`pydfcsr_gb300.beams.Beam.from_particle` and
:meth:`~pydfcsr_gb300.beams.Beam.to_particle` connect these to the GPU beam.
"""
import collections
import sys

import numpy as np

__all__ = ["Particle", "C_LIGHT", "M_ELECTRON", "E_CHARGE", "openpmd_to_bmadx_coords",
           "openpmd_to_bmadx_particles", "bmadx_particles_to_openpmd"]

# bmadx.constants: speed of light (m/s), electron rest energy (eV), elementary
# charge (C); CODATA 2018
C_LIGHT = 299792458.0
M_ELECTRON = 0.51099895000e6
E_CHARGE = 1.602176634e-19

# the fields of bmadx.structures.Particle: phase-space coordinates, then the
# position s, the reference momentum p0c (eV) and the rest energy mc2 (eV)
Particle = collections.namedtuple("Particle", "x px y py z pz s p0c mc2")


def _particle_type():
    try:
        from bmadx.structures import Particle as BmadxParticle
        return BmadxParticle
    except ImportError:
        return Particle


def openpmd_to_bmadx_coords(pmd_particle, p0c):
    """(x, px, y, py, z, pz) in bmad units from an openPMD particle group:
    transverse momenta and the momentum deviation normalised by ``p0c``
    (interfaces.py:13-39)."""
    return (pmd_particle.x, pmd_particle.px / p0c, pmd_particle.y, pmd_particle.py / p0c,
            pmd_particle.z, pmd_particle.p / p0c - 1.0)


def openpmd_to_bmadx_particles(pmd_particle, p0c, s=0.0, mc2=M_ELECTRON):
    """A bmadx ``Particle`` (or this module's stand-in) from an openPMD
    particle group (interfaces.py:40-63)."""
    return _particle_type()(*openpmd_to_bmadx_coords(pmd_particle, p0c), s=s, p0c=p0c, mc2=mc2)


def bmadx_particles_to_openpmd(particle, charge):
    """openPMD data of a bmadx ``Particle`` with numpy or torch arrays
    (interfaces.py:66-127): momenta in eV/c, the arrival time
    t = (s - z) / (c beta), status 1, equal weights summing to ``charge``,
    species electron (the only one supported).  Returns a ``ParticleGroup``
    when pmd_beamphysics is installed, else its data dict."""
    lib = sys.modules[type(particle.x).__module__]
    names = ("x", "px", "y", "py", "z", "pz")
    if lib is np:
        x, px, y, py, z, pz = (getattr(particle, k) for k in names)
    elif type(particle.x).__module__.startswith("torch"):
        x, px, y, py, z, pz = (getattr(particle, k).detach().cpu().numpy() for k in names)
    else:
        raise ValueError("Only numpy and torch Particles are supported as of now")
    p0c = particle.p0c
    p = (1 + pz) * p0c
    beta = ((p / M_ELECTRON) ** 2 / (1 + (p / M_ELECTRON) ** 2)) ** 0.5
    if not np.isclose(particle.mc2, M_ELECTRON):
        raise ValueError("only electrons are supported as of now")
    data = {"x": x, "px": px * p0c, "y": y, "py": py * p0c, "z": z,
            "pz": p0c * ((pz + 1.0) ** 2 - px ** 2 - py ** 2) ** 0.5,
            "t": (particle.s - z) / (C_LIGHT * beta),
            "status": np.ones_like(x, dtype=int),
            "weight": np.ones_like(x) * charge / len(x),
            "species": "electron"}
    try:
        from pmd_beamphysics import ParticleGroup
    except ImportError:
        return data
    return ParticleGroup(data=data)
