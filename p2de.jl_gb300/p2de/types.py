"""Parameter and method types with the names of P2DE.jl's dispatch types
(src/common/types/Solver.jl, StateParam.jl, TimeParam.jl). Method choice is by
instance type, as in the reference; to_abi() lowers a Param to the C descriptor.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

import numpy as np


# --- dimensions and equations (Solver.jl:97-121) --------------------------------------
class Dim1:
    pass


class Dim2:
    pass


@dataclass(frozen=True)
class CompressibleEulerIdealGas:
    """CompressibleEulerIdealGas{Dim2}(gamma); dim=Dim1 for CompressibleEulerIdealGas{Dim1}."""

    gamma: float = 1.4
    dim: type = Dim2


def is_dim1(equation) -> bool:
    """dim(equation) isa Dim1 (src/common/traits.jl:133-139)."""
    return getattr(equation, "dim", Dim2) is Dim1


@dataclass(frozen=True)
class KPP:
    """KPP{Dim2}() (src/math/KPP.jl): u_t + (sin u)_x + (cos u)_y = 0."""

    dim: type = Dim2


def get_gamma(equation: CompressibleEulerIdealGas) -> float:
    return equation.gamma


# --- surface / volume fluxes (Solver.jl:15-22) ----------------------------------------
class ChandrashekarFlux:
    pass


class ChandrashekarOnProjectedVal:
    pass


class LaxFriedrichsOnNodalVal:
    pass


class LaxFriedrichsOnProjectedVal:
    pass


# --- RHS types (Solver.jl:1-36) -------------------------------------------------------
@dataclass(frozen=True)
class LowOrderPositivity:
    surface_flux: Any = field(default_factory=LaxFriedrichsOnNodalVal)


@dataclass(frozen=True)
class EntropyStable:
    """FluxDiffRHS{ChandrashekarFlux}."""

    surface_flux: Any = field(default_factory=LaxFriedrichsOnProjectedVal)
    volume_flux: Any = field(default_factory=ChandrashekarFlux)


@dataclass(frozen=True)
class ESLimitedLowOrderPos:
    """LimitedDG{LOW, HIGH, ChandrashekarFlux}."""

    low_order_surface_flux: Any = field(default_factory=LaxFriedrichsOnNodalVal)
    high_order_surface_flux: Any = field(default_factory=LaxFriedrichsOnProjectedVal)
    high_order_volume_flux: Any = field(default_factory=ChandrashekarFlux)


# --- bases, entropy projection, limiters (Solver.jl:38-95) ----------------------------
class LobattoCollocation:
    pass


class GaussCollocation:
    pass


class NoEntropyProjectionLimiter:
    pass


class NodewiseScaledExtrapolation:
    pass


class NoRHSLimiter:
    pass


class NoShockCapture:
    pass


@dataclass(frozen=True)
class HennemannShockCapture:
    a: float = 0.5
    c: float = 1.8


class PositivityBound:
    pass


class PositivityAndCellEntropyBound:
    pass


class PositivityAndMinEntropyBound:
    pass


class PositivityAndRelaxedMinEntropyBound:
    pass


@dataclass(frozen=True)
class PositivityAndRelaxedCellEntropyBound:
    beta: float = 0.5


class TVDBound:
    pass


class TVDAndCellEntropyBound:
    pass


class TVDAndMinEntropyBound:
    pass


class TVDAndRelaxedMinEntropyBound:
    pass


@dataclass(frozen=True)
class TVDAndRelaxedCellEntropyBound:
    beta: float = 0.5


@dataclass(frozen=True)
class SubcellLimiter:
    bound: Any = field(default_factory=PositivityBound)
    shockcapture: Any = field(default_factory=NoShockCapture)


@dataclass(frozen=True)
class ZhangShuLimiter:
    shockcapture: Any = field(default_factory=NoShockCapture)


# --- parameters (Solver.jl:123-170) ---------------------------------------------------
@dataclass(frozen=True)
class GlobalConstant:
    POSTOL: float = 1e-14
    ZEROTOL: float = 5e-16


@dataclass(frozen=True)
class TimesteppingParameter:
    T: float
    CFL: float
    dt0: float
    t0: float = 0.0


@dataclass(frozen=True)
class LimitingParameter:
    zeta: float = 0.1
    eta: float = 0.5


@dataclass(frozen=True)
class PostprocessingParameter:
    output_interval: int = 100


@dataclass(frozen=True)
class Param:
    """Param (Solver.jl:151-170). reference_semantics and precision select the
    GB300 modes: reference_semantics=True reproduces the bound destructuring of
    limiter_utils.jl:66-70; precision is "fp64", "mixed" (FP32 flux differencing with FP32
    accumulation) or "mixed-acc64" (FP32 two-point fluxes, FP64 gather and lift)."""

    N: int
    K: tuple[int, int]
    xL: tuple[float, float]
    xR: tuple[float, float]
    global_constants: GlobalConstant
    timestepping_param: TimesteppingParameter
    limiting_param: LimitingParameter = field(default_factory=LimitingParameter)
    postprocessing_param: PostprocessingParameter = field(default_factory=PostprocessingParameter)
    equation: CompressibleEulerIdealGas = field(default_factory=CompressibleEulerIdealGas)
    approximation_basis: Any = field(default_factory=LobattoCollocation)
    rhs: Any = field(default_factory=ESLimitedLowOrderPos)
    entropyproj_limiter: Any = field(default_factory=NoEntropyProjectionLimiter)
    rhs_limiter: Any = field(default_factory=SubcellLimiter)
    reference_semantics: bool = True
    precision: str = "fp64"


def num_elements(param: Param) -> int:
    """num_elements (src/common/traits.jl:162-171): K on a Line, K[0] K[1] on quads."""
    return int(param.K) if np.isscalar(param.K) else param.K[0] * param.K[1]


def num_components(equation=None) -> int:
    """num_components (src/common/traits.jl:145-155)."""
    if isinstance(equation, KPP):
        return 1
    return 3 if is_dim1(equation) else 4


# --- boundary data and time parameters ------------------------------------------------
@dataclass
class BCData:
    """BCData{Nc} (StateParam.jl:1-7): mapP (K, Nfp) 1-based, mapI/mapO 1-based lists,
    Ival (nI, 4). mapW (reflecting walls) and mapS with xyS and the shock states
    (an oblique moving shock Dirichlet boundary) have no counterpart in BCData; they
    are what the double Mach reflection problem needs."""

    mapP: np.ndarray
    mapI: Any = ()
    mapO: Any = ()
    Ival: Any = ()
    mapW: Any = ()
    mapS: Any = ()
    xyS: Any = ()
    shock_x0: float = 0.0
    shock_inv_slope: float = 0.0
    shock_speed: float = 0.0
    shock_post: tuple = (0.0, 0.0, 0.0, 0.0)
    shock_pre: tuple = (0.0, 0.0, 0.0, 0.0)


@dataclass(frozen=True)
class TimeParam:
    """TimeParam (TimeParam.jl:1-6) without the timer."""

    t: float
    dt: float
    nstage: int


@dataclass(frozen=True)
class ErrorData:
    L1err: float
    L2err: float
    Linferr: float


@dataclass
class DataHistory:
    """DataHistory (PostprocessData.jl): snapshots of Uq and L_local."""

    Uhist: list
    Lhist: list
    thetahist: list
    thist: list
    dthist: list
