"""GB300 implementation of P2DE.jl's 2D Euler DG right-hand side and SSP-RK3 step.

The compute path is libp2de_gpu.so (hand-written CUDA for sm_103a behind the C ABI
of include/p2de.h); this package is the host-side mirror of the reference's
interface: Param and the dispatch types, initialize_DG, rhs! (rhs_bang) and
SSP33! (SSP33_bang).
"""
from . import abi, mesh, problems
from .abi import P2deError, load_library
from .mesh import MeshData, gll_rule, make_periodic, uniform_mesh
from .problems import primitive_to_conservative
from .solver import (
    Descriptor,
    HostState,
    Preallocation,
    Solver,
    State,
    StateParam,
    SSP33_bang,
    SSP33_host_loop,
    UnsupportedMethod,
    calculate_error,
    check_conservation,
    evaluate_initial_condition,
    initialize_DG,
    lower_param,
    make_descriptor,
    rhs_bang,
    ssp33_step,
)
from .types import *  # noqa: F401,F403  (the dispatch-type names of P2DE.jl)

__all__ = [
    "abi",
    "mesh",
    "problems",
    "P2deError",
    "load_library",
    "MeshData",
    "gll_rule",
    "make_periodic",
    "uniform_mesh",
    "primitive_to_conservative",
    "Descriptor",
    "HostState",
    "Preallocation",
    "Solver",
    "State",
    "StateParam",
    "SSP33_bang",
    "SSP33_host_loop",
    "UnsupportedMethod",
    "calculate_error",
    "check_conservation",
    "evaluate_initial_condition",
    "initialize_DG",
    "lower_param",
    "make_descriptor",
    "rhs_bang",
    "ssp33_step",
]
