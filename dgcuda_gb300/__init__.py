"""dgcuda_gb300 -- GB300-native RK-DG solver for 2D conservation laws.

Thin ctypes binding over the C ABI in include/dg.h.  The names mirror the
reference's host driver (src/2d/conservation/main.cu, time_integrator.cu):
``read_mesh``, ``init_conditions``, ``eval_rhs``, ``limit_c``,
``time_integrate_*``, ``eval_error_L2``, ``eval_global_lambda``; errors come
back as DGError (the reference calls exit()).  All numerics run in the native
library; there is no Python fallback -- importing fails loudly when
libdg_gb300.so is missing.
"""
from .api import (DGError, Mesh, Solver, Batch, Adjoint, Params, lib_path, load_library,  # noqa: F401
                  ADVECTION, EULER, SHALLOW_WATER, MAXWELL, SSP_RK3, RK4, RK2,
                  BC_REFLECT, BC_OUTFLOW, BC_INFLOW, BC_TRANSMISSIVE, PERIODIC, PROBLEMS,
                  n_modes, n_vars, measure_fp64_peak, probe_reciprocal, oz_table_image,
                  params_for_problem, probe_physical, probe_sqrt)
