"""kb2pi -- Python host mirror of the TwoPIScalar GPU numerics (libkb2pi).

``capi`` binds the C ABI of include/kb2pi.h; ``twopiscalar`` mirrors the
reference's problem/solution/initialize!/evolve!/measure! interface over it;
``adjoint`` holds the gradient entry point (kb_adjoint) and its loss helpers.
"""
from . import adjoint, capi  # noqa: F401
from .capi import Handle, KbError, KbParams, load_library  # noqa: F401
from .twopiscalar import (  # noqa: F401
    QFTdynamicsProblem, QFTdynamicsSolution, TwoPIScalarfile, createMeasurement, evolve, getGapMass,
    evolve_recorded, getparticlenr, initialize, lattice_orbits, load_measurearray, make_problem, measure,
    orbits_to_shells, run_simulation, save_measurearray,
)
