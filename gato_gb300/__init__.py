"""gato_gb300: GATO's Fock-operator path on GB300 (sm_103a).

The public modules mirror the reference package's (grid, operators,
hamiltonian, potentials, pseudopotentials, geometry, geometry_opt, scf,
solvers.poisson, solvers.lanczos, physics.water) with the same names and
arguments; arrays are CUDA tensors and every numerical kernel lives in the
C-ABI library libgato_cuda (include/gato.h).
"""
from .geometry import Nuclei, bond_angle, bond_length, diatomic_along_z, nuclear_repulsion, recenter
from .grid import Grid3D, inner_product, integrate, norm_sq, normalize
from .hamiltonian import Hamiltonian
from .operators import kinetic, laplacian
from .potentials import constant, harmonic_oscillator, multi_center_softened_coulomb, softened_coulomb

__all__ = [
    "Grid3D", "Hamiltonian", "Nuclei", "bond_angle", "bond_length", "constant", "diatomic_along_z",
    "harmonic_oscillator", "inner_product", "integrate", "kinetic", "laplacian",
    "multi_center_softened_coulomb", "norm_sq", "normalize", "nuclear_repulsion", "recenter",
    "softened_coulomb",
]
