"""moljax_gb300.core -- GPU-native counterpart of ``moljax.core``."""

from moljax_gb300.core.grid import Grid1D, Grid2D
from moljax_gb300.core.bc import BCType, FieldBCSpec, apply_bc
from moljax_gb300.core import fft_solvers, operators, stepping, dt_policy, model
from moljax_gb300.core.operators import LinearOp, NonlinearOp, laplacian_2d
from moljax_gb300.core.model import (MOLModel, create_gray_scott_model,
                                     create_gray_scott_periodic_fft, gray_scott_factory,
                                     create_variable_diffusion_model,
                                     create_advection_diffusion_model, create_advdiff_periodic_fft,
                                     create_fisher_kpp_model)
from moljax_gb300.core.stepping import (IntegratorType, AdaptiveResult, adaptive_integrate,
                                        adaptive_integrate_imex, imex_strang_step, imex_euler_step,
                                        integrate_imex_fixed_dt, be_step, cn_step, bdf2_step,
                                        integrate_fixed_dt, euler_step, ssprk3_step, rk4_step)
from moljax_gb300.core.dt_policy import CFLParams, PIDParams
from moljax_gb300.core.fft_solvers import (create_fft_cache, solve_helmholtz_2d,
                                           apply_diffusion_inverse_fft, fft_cn_step,
                                           laplacian_symbol_2d, fft_cn_step_3d, solve_helmholtz_3d,
                                           get_plan3d, solve_diffusion_fft_field, apply_diffusion_fft,
                                           diffusion_rhs_fft, exponential_filter_1d,
                                           exponential_filter_2d, apply_spectral_filter_interior,
                                           apply_spectral_filter_field, apply_spectral_filter_state,
                                           create_fft_cache_1d, solve_helmholtz_1d,
                                           build_wavenumbers_2d, fft_cn_advdiff_1d, imex_advdiff_1d,
                                           gray_scott_strang_exp, gray_scott_rk4_spectral)
from moljax_gb300.core.utils import StatusCode
from moljax_gb300.core import fft_integrators, fft_operators
from moljax_gb300.core.fft_integrators import (etdrk4_gray_scott, etdrk4_step, etd_integrate, etd1_step,
                                               etd2_step, diffusion_only_etd1, NativeNonlinear,
                                               etd_integrate_model, etd_adaptive_integrate,
                                               batched_fft_matvec, batched_fft_solve,
                                               batched_fft_exp_matvec, stacked_fft_solve_shared_op)
from moljax_gb300.core.fft_operators import (DiffusionOperator, AdvectionDiffusionOperator,
                                              SpectralBounds, exact_cfl_dt)
from moljax_gb300.core import newton_krylov, preconditioners
from moljax_gb300.core.newton_krylov import (NKParams, NKStats, newton_krylov_solve,
                                             integrate_implicit_vardiff)
from moljax_gb300.core.preconditioners import (DiffusionPreconditioner, IdentityPreconditioner,
                                               BlockJacobiPreconditioner, FFTDiffusionPreconditioner,
                                               FFTAdvectionDiffusionPreconditioner, PrecondContext)
from moljax_gb300.core import reactor, stencil1d
from moljax_gb300.core.operators import (laplacian_1d, gradient_1d, d1_upwind_1d, d1_upwind_2d,
                                        d1_central_2d)
from moljax_gb300.core.utils import scaled_error_norm, is_finite
from moljax_gb300.core.dt_policy import propose_dt, implicit_robustness_dt, compute_error_order
from moljax_gb300.core import fft_nonperiodic
from moljax_gb300.core.fft_nonperiodic import (dst_I_fast, idst_I_fast, laplacian_symbol_dirichlet,
                                               create_nonperiodic_fft_cache,
                                               solve_poisson_dirichlet, solve_helmholtz_dirichlet,
                                               etd1_dirichlet, laplacian_symbol_neumann,
                                               solve_poisson_neumann, solve_helmholtz_neumann,
                                               etd1_neumann, check_compatibility_neumann,
                                               project_to_compatible)
from moljax_gb300.core import state, variable_coeff
from moljax_gb300.core.state import (tree_add, tree_sub, tree_scale, tree_axpy, tree_zeros_like,
                                     tree_ones_like, tree_norm2, tree_norm_inf, tree_vdot,
                                     flatten_to_vec, unflatten_from_vec, state_total_size,
                                     state_interior_size, create_state_from_interior,
                                     get_interior_state)
from moljax_gb300.core.variable_coeff import apply_variable_diffusion_2d
from moljax_gb300.core.operators import (d2_central_1d, d2_central_2d, d1_central_1d, op_sum,
                                        state_zero_like, make_diffusion_op_1d, make_diffusion_op_2d,
                                        make_advection_op_1d, make_advection_op_2d, make_reaction_op,
                                        fd_laplacian_symbol_1d, fd_laplacian_symbol_2d,
                                        gray_scott_reaction_op, fisher_kpp_reaction_op)
from moljax_gb300.core.stepping import (AdaptiveState, estimate_error_doubling,
                                        estimate_error_implicit, estimate_error_imex_doubling,
                                        step_explicit, step_explicit_with_error, imex_ssprk2_step)
from moljax_gb300.core.newton_krylov import create_implicit_residual, create_bdf2_residual
from moljax_gb300.core.preconditioners import (create_gray_scott_preconditioner,
                                               create_advdiff_preconditioner,
                                               create_diffusion_preconditioner,
                                               create_fft_preconditioner,
                                               create_gray_scott_fft_preconditioner,
                                               create_advdiff_fft_preconditioner)
from moljax_gb300.core.dt_policy import estimate_reaction_stiffness
from moljax_gb300.core.fft_operators import FFTLinearOperator
from moljax_gb300.core.fft_integrators import ETDStepResult
from moljax_gb300.core import batch
from moljax_gb300.core.batch import GrayScottBatch, GrayScottProblem, adaptive_integrate_imex_batch
from moljax_gb300.core.fft_solvers import gray_scott_cn_newton
from moljax_gb300.core.operators import make_kinetics_op
