"""marinehydro_gb300 -- GB300 (sm_103a) implementation of MarineHydro.jl's dense-BEM hot path.

The Python surface mirrors the reference's Julia API; assembly, dense solves and
the frequency sweep run in libmarinehydro_cuda.so (hand-written CUDA, FP64 plain
path) behind the C-ABI declared in include/marinehydro_gb300.h.  The directory
name is not a Python identifier; load it with ``load_package()`` below or
``importlib`` under the name ``marinehydro_gb300``.
"""
from ._lib import (Context, MarineHydroError, default_context, load as load_library)  # noqa: F401
from .api import (airy_bc, airy_pressure, assemble_matrices, autotune, load_tile_table, assemble_matrix_wu, batch_hydrodynamic_coefficients,  # noqa
                  calculate_radiation_forces,
                  compute_bc, compute_hydrodynamic_coefficients, excitation_force, froude_krylov_force,
                  gpu_linsolve, hydro_gradient, hydro_vjp, hydrodynamic_coefficients, hydrodynamic_coefficients_derivative, load_surrogate, set_surrogate, set_surrogate_judge, surrogate_judge_report, surrogate_wave_terms, train_surrogate, integrate_pressure, linsolve, linsolve_adjoint,
                  problems_from_data, radiation_bc, solve, solve_linear, solve_problem, solve_pullback)
from .bodies import FloatingBody, combine_floatingbodies, rotational_dofs, translational_dofs  # noqa: F401
from .formulations import (BEMFormulation, DelhommeauRankine, DelhommeauRankineReflected, DirectBEM,  # noqa: F401
                           ExactGuevelDelhommeau, GFWu, GreensFunction, IndirectBEM, Rankine, RankineReflected,
                           RankineReflectedNegative, SurrogateDelhommeau, bem_formulation, default_greens_functions, gf_flags, is_direct,
                           partition_greens_functions)
from .meshes import (Mesh, StaticArraysMesh, barge_mesh, combine_meshes, config1_hemisphere,  # noqa: F401
                     config2_cylinder, disc_lid_mesh, face_fields, face_fields_jacobian, hemisphere_mesh, random_body, smesh, tiny_static_mesh, vertical_cylinder_mesh)
from .mesh_io import mesh_from_arrays, mesh_from_capytaine, read_gdf, write_gdf  # noqa: F401
from .problems import (SETTINGS, DiffractionProblem, DiffractionResult, RadiationProblem,  # noqa: F401
                       RadiationResult, added_mass, compute_encountered_values, compute_wavenumber,
                       diffraction_force, make_result, radiation_coefficients, radiation_damping, remake, set_g,
                       set_rho)

__all__ = [n for n in dir() if not n.startswith("_")]
