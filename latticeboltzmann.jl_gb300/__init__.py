"""latticeboltzmann.jl_gb300 -- the collide-stream hot path of LatticeBoltzmann.jl on GB300.

The reference's host layer (quadratures, problems, initial conditions, collision-model and
boundary-condition descriptors, processing methods and the simulate loop) is mirrored here
in Python with the reference's names; the per-step work runs in liblbm_gb300.so, hand-written
CUDA for sm_103a behind the C ABI of include/lbm_gb300.h.  There is no CPU path: without the
library every simulation call raises.

The directory name is not a Python identifier, so load the package by path, e.g.

    import importlib.util, sys
    spec = importlib.util.spec_from_file_location(
        "latticeboltzmann_gb300", "<repo>/latticeboltzmann.jl_gb300/__init__.py",
        submodule_search_locations=["<repo>/latticeboltzmann.jl_gb300"])
    lbm = importlib.util.module_from_spec(spec); sys.modules[spec.name] = lbm
    spec.loader.exec_module(lbm)
"""
from .quadratures import (Quadrature, D2Q4, D2Q5, D2Q9, D2Q13, D2Q17, D2Q21, D2Q37, Quadratures, dimension,
                          opposite, order)
from .kinetics import (hermite, equilibrium_coefficient, equilibrium, equilibrium_, density, velocity, pressure,
                       temperature, deviatoric_tensor, momentum_flux)
from .boundary_conditions import BoundaryCondition, BounceBack, MovingWall, North, East, South, West
from .collision_models import (CollisionModel, SRT, TRT, TRT_Λ, MRT, IterativeInitializationCollisionModel,
                               make_collision_model)
from .problems import (FluidFlowProblem, TaylorGreenVortex, TGV, PoiseuilleFlow, CouetteFlow, DecayingShearFlow,
                       LidDrivenCavityFlow, LinearizedThermalDiffusion, LinearizedTransverseShearWave, ShearWave,
                       problem_range, delta_t, delta_x, viscosity, lattice_viscosity, has_external_force,
                       boundary_conditions, lattice_velocity, lattice_density, lattice_pressure, lattice_temperature,
                       lattice_force_field, analytic_fields, decay_time, node_grid)
from .initial_conditions import (InitializationStrategy, ZeroVelocityInitialCondition, AnalyticalEquilibrium, initial_fields,
                                 AnalyticalEquilibriumAndOffEquilibrium, ConstantDensity, AnalyticalVelocityAndStress,
                                 AnalyticalVelocity, IterativeInitializationMeiEtAl, IterativeInitialization,
                                 initialize)
from .processing_methods import (ProcessingMethod, TrackHydrodynamicErrors, CompareWithAnalyticalSolution,
                                 ProcessIterativeInitialization, TakeSnapshots, NoProcessing, StopCriteriaFor,
                                 NoStoppingCriteria, MeanVelocityStoppingCriteria, VelocityConvergenceStoppingCriteria,
                                 DensityConvergence, TrackRow, CompareRow, track_errors)
from .device import DeviceLattice, DeviceBatch
from .model import (LatticeBoltzmannModel, simulate, simulate_model, simulate_batch, run_steps, collide, stream,
                    apply)
from . import build_native
from .studies import (tgv_instances, run_tgv_study, convergence_order, trt_sweep_points, julia_range,
                      build_trt_sweep_models, run_trt_sweep, build_shear_wave_study_models, run_shear_wave_study,
                      SWEEP_COLUMNS, trt_sweep_table, save_sweep_table, load_sweep_table, sweep_error_grid)
from .adjoint import AdjointProblem, divergence_free_field, trt_magic, magic_total_derivative, LBMLoss

StopCriteria = StopCriteriaFor


def build(verbose: bool = False) -> str:
    """Compile liblbm_gb300.so for sm_103a (in-tree) and return its path."""
    return build_native.build(verbose=verbose)


def library_path() -> str:
    return build_native.LIB
