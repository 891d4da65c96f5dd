"""GB300 (sm_103a) stochastic-Galerkin hot path of ExtendableASGFEM.jl.

Host-side mirror of the reference API (Python names for the Julia ones,
``solve!`` -> ``solve``) over the C ABI of libsgfem.so (include/sgfem.h).
The directory name follows the Julia package naming; import it through
``load_package()`` in ``__graft_entry__`` or by path.
"""
from . import _lib
from ._lib import FP32, FP64, MIXED, PREC_CHOLESKY, PREC_JACOBI, PREC_LATTICE, PREC_NONE, SGError, cholesky_host_solve
from .adjoint import MeanQoI
from .batch import SGBatch, config4_problems, splitmix64
from .coefficients import StochasticCoefficientCosinus
from .estimate import estimate, estimate_equilibration, extension_couplings
from .fem import (H1Pk, assemble_convection, assemble_laplacian, assemble_pce_rhs, assemble_rhs, assemble_stiffness,
                  assemble_stiffness_gpu, assemble_rhs_gpu, assemble_pce_rhs_gpu, assemble_laplacian_gpu,
                  assemble_convection_gpu,
                  assemble_stiffness_nodal_mean, box_functional, line_rule, pce_lambda, perturbed_unit_square_mesh,
                  triangle_rule, unit_square_mesh)
from .modelproblems import (AbstractModelProblem, LogTransformedPoissonProblemPrimal, PoissonProblemPrimal, SGOperator,
                            assemble, solve)
from .mopcontrol import (add_boundary_modes, classify_modes, generate_multiindices, get_neighbours,
                         prepare_multi_indices, stochastic_marking, top_weight_multiindices,
                         total_degree_multiindices)
from .orthopolys import HermitePolynomials, LegendrePolynomials, ONBasis
from .sampling_error import SampleProblems, calculate_sampling_error, evaluate_samples
from .sgfevector import SGFEVector
from .tensorizedbasis import TensorizedBasis, coupling_matrix

__all__ = [
    "FP32", "FP64", "MIXED", "PREC_CHOLESKY", "PREC_JACOBI", "PREC_LATTICE", "PREC_NONE", "SGError", "MeanQoI", "SGBatch",
    "config4_problems", "splitmix64",
    "assemble_stiffness_nodal_mean", "assemble_stiffness_gpu", "box_functional",
    "StochasticCoefficientCosinus", "estimate", "extension_couplings", "H1Pk", "assemble_convection",
    "assemble_laplacian", "assemble_pce_rhs", "assemble_rhs", "assemble_stiffness", "line_rule", "pce_lambda",
    "triangle_rule", "unit_square_mesh", "perturbed_unit_square_mesh", "cholesky_host_solve", "AbstractModelProblem", "LogTransformedPoissonProblemPrimal",
    "PoissonProblemPrimal", "SGOperator", "assemble", "solve",
    "add_boundary_modes", "classify_modes", "generate_multiindices", "get_neighbours", "prepare_multi_indices",
    "stochastic_marking", "top_weight_multiindices", "total_degree_multiindices", "HermitePolynomials",
    "LegendrePolynomials", "ONBasis", "SampleProblems", "calculate_sampling_error", "evaluate_samples",
    "SGFEVector", "TensorizedBasis", "coupling_matrix",
]
