"""biblbm_gb300: the coupled immersed-boundary lattice-Boltzmann time step of
niclasberg/biblbm (Palabos + fsi), rebuilt for one GB300 (sm_103a).

The compute path is the CUDA library ``lib/libbib_gb300.so`` behind the C ABI of
``include/bib/bib.h``; this package is its host-side Python mirror.
"""
from .api import (COLLISION, DIRAC, MODEL, STORAGE, WALL, Batch, CapsuleParameters, Context,
                  ImmersedBoundaryDynamics3D, Lattice, MorsePotential, ParticleShapeLibrary, RBCParameters,
                  RBCShapeInitializer, create_particles, grow_particles, initial_distribution, place_particle,
                  SpringPotential, lattice_params, membrane_params, taylor_deformation)
from ._lib import BibError, LIB_PATH

__all__ = [
    "Batch", "BibError", "CapsuleParameters", "COLLISION", "Context", "DIRAC", "ImmersedBoundaryDynamics3D", "Lattice",
    "LIB_PATH", "MODEL", "MorsePotential", "ParticleShapeLibrary", "RBCParameters", "RBCShapeInitializer", "SpringPotential", "STORAGE",
    "WALL", "create_particles", "grow_particles", "initial_distribution", "lattice_params", "place_particle",
    "membrane_params", "taylor_deformation",
]
