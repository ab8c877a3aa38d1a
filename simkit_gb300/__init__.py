"""simkit_gb300: GB300-native backward-Euler stable neo-Hookean FEM path.

A drop-in for the hot path of otmanon/simkit: the same Python signatures for
the stable neo-Hookean energy tiers, deformation_jacobian, volume,
psd_project, backtracking_line_search, newton_solver, backward_euler and bdf2, with
the arithmetic in hand-written sm_103a CUDA kernels behind a ctypes C ABI
(include/simkit_gb300.h).  ``BESolver`` runs whole backward-Euler steps on
the device.
"""

from .beams import BeamSpec, beam_batch, beam_large_jittered, beam_small_steady, make_beam  # noqa: F401

_API = {
    "stable_neo_hookean_energy_element_F", "stable_neo_hookean_gradient_element_F",
    "stable_neo_hookean_hessian_element_F", "stable_neo_hookean_energy_x", "stable_neo_hookean_gradient_x",
    "stable_neo_hookean_hessian_x", "stable_neo_hookean_energy", "stable_neo_hookean_gradient",
    "stable_neo_hookean_hessian", "psd_project", "deformation_jacobian", "volume", "backtracking_line_search",
    "newton_solver", "backward_euler", "bdf2", "solve_sparse", "BlockMatrix", "DeformationJacobian",
    "macklin_mueller_neo_hookean_energy_element_F", "macklin_mueller_neo_hookean_gradient_element_F",
    "macklin_mueller_neo_hookean_hessian_element_F", "macklin_mueller_neo_hookean_energy_x",
    "macklin_mueller_neo_hookean_gradient_x", "macklin_mueller_neo_hookean_hessian_x",
    "macklin_mueller_neo_hookean_energy", "macklin_mueller_neo_hookean_gradient",
    "macklin_mueller_neo_hookean_hessian", "arap_energy_element_F", "arap_gradient_element_F",
    "arap_hessian_element_F", "arap_energy_x", "arap_gradient_x", "arap_hessian_x", "arap_energy",
    "arap_gradient", "arap_hessian", "fcr_energy_element_F", "fcr_gradient_element_F",
    "fcr_hessian_element_F", "fcr_energy_x", "fcr_gradient_x", "fcr_hessian_x", "fcr_energy",
    "fcr_gradient", "fcr_hessian", "stable_neo_hookean_energy_u", "stable_neo_hookean_gradient_u",
    "stable_neo_hookean_hessian_u", "macklin_mueller_neo_hookean_energy_u", "macklin_mueller_neo_hookean_gradient_u",
    "macklin_mueller_neo_hookean_hessian_u", "arap_energy_u", "arap_gradient_u", "arap_hessian_u", "fcr_energy_u",
    "fcr_gradient_u", "fcr_hessian_u", "elastic_energy_u", "elastic_gradient_u", "elastic_hessian_u",
    "linear_elasticity_energy_element_F", "linear_elasticity_gradient_element_F",
    "linear_elasticity_hessian_element_F", "linear_elasticity_energy_x", "linear_elasticity_gradient_x",
    "linear_elasticity_hessian_x", "linear_elasticity_energy_u", "linear_elasticity_gradient_u",
    "linear_elasticity_hessian_u", "linear_elasticity_energy", "linear_elasticity_gradient",
    "linear_elasticity_hessian", "elastic_energy_element_F", "elastic_gradient_element_F",
    "elastic_hessian_element_F", "elastic_energy_x", "elastic_gradient_x", "elastic_hessian_x",
    "elastic_energy", "elastic_gradient", "elastic_hessian", "contact_springs_plane_energy",
    "contact_springs_plane_gradient", "contact_springs_plane_hessian", "ElasticPotential",
}


def __getattr__(name):
    # torch and the CUDA library load on first use of an entry point
    if name in _API:
        from . import api
        return getattr(api, name)
    if name == "BESolver":
        from .solver import BESolver
        return BESolver
    if name == "TetMesh":
        from .mesh import TetMesh
        return TetMesh
    if name == "BatchedBESolver":
        from .batched import BatchedBESolver
        return BatchedBESolver
    raise AttributeError(name)
