"""GB300-native semi-discrete residual for StableSpectralElements.jl
(successor of CLOUD.jl): host-side operator construction mirroring the
reference's API plus the C-ABI CUDA library ``libsse_gb300.so``.

The directory name contains a dot, so it is loaded as the module
``cloud_jl_gb300`` (see ``__graft_entry__.load_package``).
"""
from . import (abi, build, flops_model, gb300, jld2, mesh, objectives, polynomials, reference,  # noqa: F401
               setups, solver, timestepping)
from .gb300 import (GB300Solver, ODEProblem, SSEError, load_library,  # noqa: F401
                    semi_discrete_residual, semidiscretize)
from .mesh import spatial_discretization, uniform_periodic_mesh, warp_mesh  # noqa: F401
from .reference import reference_approximation  # noqa: F401
from .timestepping import l2_error, solve  # noqa: F401
from .solver import (CentralNumericalFlux, EntropyConservativeFlux,  # noqa: F401
                     EntropyConservativeNumericalFlux, EulerEquations, FluxDifferencingForm,
                     HostArrays, LaxFriedrichsNumericalFlux, LinearAdvectionEquation,
                     StandardForm, initialize)
