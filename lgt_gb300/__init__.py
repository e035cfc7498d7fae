"""lgt_gb300: exact diagonalisation of the U(1) lattice gauge theory of
NoaFeldman/LGT on a GB300 GPU (sm_103a), behind the reference's own entry
points (finite_ed.jl).  All compute runs in the CUDA library liblgted.so
(include/lgt_ed.h); there is no CPU fallback."""
from .ed import (HPSI_KERNELS, Basis, Hamiltonian, KeyDict, build_basis, build_hamiltonian,
                 encode, find_ground_states, find_ground_state_measured,
                 evolve_ED, find_ground_state, ite_ground_state_ED, measure_ED,
                 staggered_charges, staggered_product_state, string_charges, string_state)
from ._capi import LgtError, NotConverged

__all__ = [
    "HPSI_KERNELS", "Basis", "Hamiltonian", "KeyDict", "build_basis", "build_hamiltonian", "encode",
    "evolve_ED", "find_ground_state", "find_ground_state_measured", "find_ground_states",
    "ite_ground_state_ED", "measure_ED", "staggered_charges",
    "staggered_product_state", "string_charges", "string_state", "LgtError", "NotConverged",
]
