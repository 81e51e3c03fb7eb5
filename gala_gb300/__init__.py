"""gala_gb300: GB300-native orbit integration behind gala's integrate_orbit API.

The public surface mirrors gala's: potential classes
(``gala_gb300.potential``), ``Hamiltonian`` with ``integrate_orbit``, frames,
``Orbit`` / ``PhaseSpacePosition`` (with gala's HDF5 files, ``gala_gb300.hdf5``),
potential YAML files (``gala_gb300.potential_io``) and
``parse_time_specification``.  All
evaluation and integration runs in the CUDA library built from
``gala_gb300/csrc`` (C ABI: include/gala_gb300.h).
"""
from . import hdf5, potential_io, units
from .dynamics import Orbit, PhaseSpacePosition
from .hamiltonian import ConstantRotatingFrame, Hamiltonian, StaticFrame
from .integrate import (DOPRI853Integrator, LeapfrogIntegrator, Ruth4Integrator, get_integrator,
                        parse_time_specification)
from .potential import (CCompositePotential, CompositePotential, HernquistPotential, KeplerPotential,
                        MilkyWayPotential, MiyamotoNagaiPotential, NFWPotential, NullPotential,
                        PlummerPotential, SCFPotential)

__all__ = [
    "hdf5", "potential_io", "units", "Orbit", "PhaseSpacePosition", "Hamiltonian", "StaticFrame", "ConstantRotatingFrame",
    "LeapfrogIntegrator", "Ruth4Integrator", "DOPRI853Integrator", "get_integrator", "parse_time_specification",
    "CCompositePotential", "CompositePotential", "HernquistPotential", "KeplerPotential", "MilkyWayPotential",
    "MiyamotoNagaiPotential", "NFWPotential", "NullPotential", "PlummerPotential", "SCFPotential",
]


def load_library():
    """Build (if needed) and load the CUDA library; returns the ctypes handle."""
    from . import _abi

    return _abi.load()
