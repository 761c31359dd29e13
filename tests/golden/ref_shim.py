"""Import pyDFCSR_2D from a read-only checkout with stub modules for absent deps.

Used only by ``make_golden.py`` in a container that holds the reference source
tree.  Nothing at test, smoke or bench time imports this module: the fixtures
it helps produce are committed as ``.npz`` files next to it.

The reference's hot-path modules (``deposit.py``, ``interp3D.py``,
``interp1D.py``, ``lattice.py``, ``CSR.py``) import several packages that are
not needed for the arithmetic of the wake path (numba, bmadx, h5py, mpi4py,
yaml, distgen, pmd_beamphysics, matplotlib).  This shim installs minimal
stand-ins so the modules import unchanged:

* ``numba.jit`` / ``jitclass`` become identity decorators and ``prange`` is
  ``range`` - the numba loops then run as ordinary Python with the same IEEE
  double arithmetic (numba does not contract a*b+c into FMA without fastmath);
* the other packages become empty modules carrying the few names imported;
* ``np.trapz`` is aliased to ``np.trapezoid`` (removed in numpy 2).
"""
import sys
import types

import numpy as np


def _identity_decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(f):
        return f
    return wrap


class _AnyIndex:
    def __getitem__(self, item):
        return self

    def __call__(self, *a, **k):
        return self


def _module(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    sys.modules[name] = m
    return m


class _Dummy:
    def __init__(self, *a, **k):
        self.args = a
        self.kwargs = k


def install(reference_root):
    """Install the stubs and put ``reference_root`` on sys.path."""
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    sys.dont_write_bytecode = True

    numba = _module("numba", jit=_identity_decorator, njit=_identity_decorator,
                    prange=range, double=_AnyIndex(), float64=_AnyIndex(),
                    int64=_AnyIndex())
    exp = _module("numba.experimental", jitclass=_identity_decorator)
    numba.experimental = exp

    bmadx = _module("bmadx", Drift=_Dummy, SBend=_Dummy, Quadrupole=_Dummy,
                    Sextupole=_Dummy, Particle=_Dummy, M_ELECTRON=0.51099895e6,
                    track_element=lambda p, e: p)
    bmadx.constants = _module("bmadx.constants", C_LIGHT=299792458.0,
                              M_ELECTRON=0.51099895e6,
                              E_CHARGE=1.602176634e-19)
    bmadx.structures = _module("bmadx.structures", Particle=_Dummy)
    _module("h5py", File=_Dummy)
    mpi = _module("mpi4py")
    mpi.MPI = _module("mpi4py.MPI", COMM_WORLD=None, DOUBLE=None)
    _module("yaml", load=None, dump=None, SafeLoader=object, Loader=object,
            SafeDumper=object, Dumper=object,
            resolver=types.SimpleNamespace(BaseResolver=types.SimpleNamespace(
                DEFAULT_MAPPING_TAG="tag:yaml.org,2002:map")))
    _module("distgen", Generator=_Dummy)
    _module("pmd_beamphysics", ParticleGroup=_Dummy)
    mpl = _module("matplotlib", cm=None)
    mpl.pyplot = _module("matplotlib.pyplot")
    mpl.cm = _module("matplotlib.cm")

    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
    import pyDFCSR_2D.deposit as deposit  # noqa: F401
    import pyDFCSR_2D.interp3D as interp3D  # noqa: F401
    import pyDFCSR_2D.interp1D as interp1D  # noqa: F401
    import pyDFCSR_2D.lattice as lattice  # noqa: F401
    import pyDFCSR_2D.CSR as CSR  # noqa: F401
    import pyDFCSR_2D.r_gen6 as r_gen6  # noqa: F401
    return types.SimpleNamespace(deposit=deposit, interp3D=interp3D,
                                 interp1D=interp1D, lattice=lattice, CSR=CSR,
                                 r_gen6=r_gen6)
