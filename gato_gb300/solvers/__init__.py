from .lanczos import LanczosResult, default_krylov_dim, lanczos
from .poisson import hartree_energy, hartree_potential

__all__ = ["LanczosResult", "default_krylov_dim", "hartree_energy", "hartree_potential", "lanczos"]
