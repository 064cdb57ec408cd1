"""Initial and boundary data of the benchmark problems (the drivers of the solve).

Kelvin-Helmholtz (periodic), double Mach reflection (inflow, reflecting wall, outflow,
moving-shock top boundary), four-quadrant Riemann problems (outflow) and the
isentropic vortex of test/test_smoke.jl:6-20 (periodic). Each problem returns a
Param plus the initial_condition / initial_boundary_conditions callables that
initialize_DG takes. Noise is drawn from numpy's PCG64 with a fixed seed, so the
same Uq is fed to every implementation.
"""
from __future__ import annotations

import math
from dataclasses import replace

import numpy as np

from .mesh import MeshData, make_periodic
from .types import (
    BCData,
    CompressibleEulerIdealGas,
    ESLimitedLowOrderPos,
    GlobalConstant,
    LimitingParameter,
    LobattoCollocation,
    NoEntropyProjectionLimiter,
    Param,
    PositivityAndCellEntropyBound,
    PostprocessingParameter,
    SubcellLimiter,
    TimesteppingParameter,
)


def primitive_to_conservative(equation, prim) -> np.ndarray:
    """primitive_to_conservative(::CompressibleIdealGas{Dim2}) (compressible_Navier_Stokes.jl:9-16),
    vectorised: (rho, u, v, p) arrays -> (..., 4)."""
    gamma = equation.gamma
    rho, u, v, p = (np.asarray(a, dtype=np.float64) for a in prim)
    rho, u, v, p = np.broadcast_arrays(rho, u, v, p)
    E = p / (gamma - 1) + 0.5 * rho * (u**2 + v**2)
    return np.stack([rho, rho * u, rho * v, E], axis=-1)


def default_param(N, K, xL, xR, T, CFL=0.5, dt0=None, bound=None, precision="fp64", reference_semantics=True,
                  output_interval=100000, rhs_limiter=None, approximation_basis=None, entropyproj_limiter=None):
    """Param with the smoke test's constants (test/test_smoke.jl:57-67): POSTOL=1e-14,
    ZEROTOL=5e-16, zeta=0.1, eta=0.5; ESLimitedLowOrderPos(LaxFriedrichsOnNodalVal,
    LaxFriedrichsOnProjectedVal), NoEntropyProjectionLimiter, SubcellLimiter(bound) unless
    rhs_limiter is given. dt0 defaults to T so that the positivity CFL governs the step."""
    if rhs_limiter is None:
        rhs_limiter = SubcellLimiter(bound=bound if bound is not None else PositivityAndCellEntropyBound())
    return Param(
        N=N,
        K=tuple(K),
        xL=tuple(xL),
        xR=tuple(xR),
        global_constants=GlobalConstant(POSTOL=1e-14, ZEROTOL=5e-16),
        timestepping_param=TimesteppingParameter(T=T, CFL=CFL, dt0=T if dt0 is None else dt0, t0=0.0),
        limiting_param=LimitingParameter(zeta=0.1, eta=0.5),
        postprocessing_param=PostprocessingParameter(output_interval=output_interval),
        equation=CompressibleEulerIdealGas(1.4),
        rhs=ESLimitedLowOrderPos(),
        rhs_limiter=rhs_limiter,
        approximation_basis=approximation_basis if approximation_basis is not None else LobattoCollocation(),
        entropyproj_limiter=entropyproj_limiter if entropyproj_limiter is not None else NoEntropyProjectionLimiter(),
        reference_semantics=reference_semantics,
        precision=precision,
    )


def periodic_bc(param, md: MeshData) -> BCData:
    """initial_boundary_conditions of test/test_smoke.jl:22-36: make_periodic, no mapI/mapO."""
    return BCData(mapP=make_periodic(md).mapP)


def outflow_bc(param, md: MeshData) -> BCData:
    """All boundary face nodes are outflow (mapO); mapP maps them to themselves."""
    return BCData(mapP=md.mapP, mapO=md.mapB)


# --- Kelvin-Helmholtz -----------------------------------------------------------------
def kelvin_helmholtz(N=3, Kx=32, Ky=32, T=0.1, seed=0, noise=1e-3, **kw):
    """rho=2, u=0.5 for |y-0.5|<0.25, else rho=1, u=-0.5; p=2.5; v=0.1 sin(4 pi x);
    uniform noise of amplitude `noise` on u and v; periodic [0,1]^2."""
    param = default_param(N, (Kx, Ky), (0.0, 0.0), (1.0, 1.0), T, **kw)

    def initial_condition(param, x, y):
        rng = np.random.Generator(np.random.PCG64(seed))
        du = rng.uniform(-noise, noise, size=x.shape)
        dv = rng.uniform(-noise, noise, size=x.shape)
        inner = np.abs(y - 0.5) < 0.25
        rho = np.where(inner, 2.0, 1.0)
        u = np.where(inner, 0.5, -0.5) + du
        v = 0.1 * np.sin(4.0 * np.pi * x) + dv
        p = np.full_like(x, 2.5)
        return primitive_to_conservative(param.equation, (rho, u, v, p))

    return param, initial_condition, periodic_bc


# --- double Mach reflection -----------------------------------------------------------
DMR_PRE = (1.4, 0.0, 0.0, 1.0)
DMR_POST = (8.0, 8.25 * math.cos(math.pi / 6), -8.25 * math.sin(math.pi / 6), 116.5)
DMR_X0 = 1.0 / 6.0


def double_mach_reflection(N=3, Kx=480, Ky=120, T=0.2, **kw):
    """Mach-10 shock at 60 degrees from x = 1/6 on [0,4]x[0,1]; reflecting wall for
    x > 1/6 at y = 0, post-shock inflow for x < 1/6 at y = 0 and at x = 0, outflow at
    x = 4, exact moving-shock data at y = 1 (shock at x = 1/6 + (y + 20 t)/sqrt(3))."""
    param = default_param(N, (Kx, Ky), (0.0, 0.0), (4.0, 1.0), T, **kw)
    eq = param.equation
    post = primitive_to_conservative(eq, DMR_POST)
    pre = primitive_to_conservative(eq, DMR_PRE)
    inv_slope = 1.0 / math.sqrt(3.0)

    def initial_condition(param, x, y):
        behind = x < DMR_X0 + y * inv_slope
        return np.where(behind[..., None], post, pre)

    def boundary(param, md: MeshData) -> BCData:
        xf, yf = md.xf.ravel(), md.yf.ravel()
        bottom, top = md.sides["bottom"], md.sides["top"]
        left, right = md.sides["left"], md.sides["right"]
        b_in = bottom[xf[bottom - 1] < DMR_X0]
        b_wall = bottom[xf[bottom - 1] >= DMR_X0]
        mapI = np.concatenate([left, b_in])
        Ival = np.tile(post, (mapI.size, 1))
        xyS = np.stack([xf[top - 1], yf[top - 1]], axis=1)
        return BCData(
            mapP=md.mapP,
            mapI=mapI,
            Ival=Ival,
            mapO=right,
            mapW=b_wall,
            mapS=top,
            xyS=xyS,
            shock_x0=DMR_X0,
            shock_inv_slope=inv_slope,
            shock_speed=20.0,
            shock_post=tuple(post),
            shock_pre=tuple(pre),
        )

    return param, initial_condition, boundary


# --- four-quadrant Riemann problem ----------------------------------------------------
def riemann_quadrant_states(seed: int) -> np.ndarray:
    """(4, 4) primitive states (rho, u, v, p) of quadrants NE, NW, SW, SE:
    rho ~ U[0.1, 2], p ~ U[0.02, 2], u, v ~ U[-1, 1]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rho = rng.uniform(0.1, 2.0, 4)
    p = rng.uniform(0.02, 2.0, 4)
    u = rng.uniform(-1.0, 1.0, 4)
    v = rng.uniform(-1.0, 1.0, 4)
    return np.stack([rho, u, v, p], axis=1)


def riemann2d(N=3, Kx=64, Ky=64, T=0.2, seed=0, **kw):
    """Four-quadrant Riemann problem on [0,1]^2 with outflow boundaries."""
    param = default_param(N, (Kx, Ky), (0.0, 0.0), (1.0, 1.0), T, **kw)
    st = riemann_quadrant_states(seed)

    def initial_condition(param, x, y):
        q = np.where(x >= 0.5, np.where(y >= 0.5, 0, 3), np.where(y >= 0.5, 1, 2))
        prim = tuple(st[q, c] for c in range(4))
        return primitive_to_conservative(param.equation, prim)

    return param, initial_condition, outflow_bc


# --- isentropic vortex ----------------------------------------------------------------
def sedov_exact(gamma=1.4, r_ini=4 * 3 / 80):
    """exact_sol of examples/2D/sedov.jl:9-20 (the initial data): rho 1, at rest, pressure
    (gamma - 1) / (pi r_ini^2) inside r < r_ini (r_ini = 12 / 80 there, whatever the mesh)
    and 1e-5 outside."""

    def exact_sol(equation, x, y, t):
        r = np.sqrt(np.asarray(x) ** 2 + np.asarray(y) ** 2)
        p = np.where(r < r_ini, (gamma - 1) * 1 / np.pi / r_ini / r_ini, 1e-5)
        one = np.ones_like(r)
        return (one, 0 * one, 0 * one, p)

    return exact_sol


def sedov(N=3, Kx=80, Ky=80, T=1.0, rhs_limiter=None, reference_semantics=True, **kw):
    """examples/2D/sedov.jl:42-55: periodic [-1.5, 1.5]^2, GaussCollocation with
    NodewiseScaledExtrapolation, ESLimitedLowOrderPos(LaxFriedrichsOnProjectedVal,
    LaxFriedrichsOnProjectedVal), ZhangShuLimiter, zeta 0.1, eta 0.1, CFL 0.5, dt0 1e-3."""
    from dataclasses import replace

    from .types import GaussCollocation, LaxFriedrichsOnProjectedVal, NodewiseScaledExtrapolation, ZhangShuLimiter

    kw.setdefault("CFL", 0.5)
    kw.setdefault("dt0", 1e-3)
    param = default_param(N, (Kx, Ky), (-1.5, -1.5), (1.5, 1.5), T,
                          rhs_limiter=rhs_limiter if rhs_limiter is not None else ZhangShuLimiter(),
                          reference_semantics=reference_semantics, approximation_basis=GaussCollocation(),
                          entropyproj_limiter=NodewiseScaledExtrapolation(), **kw)
    param = replace(param, limiting_param=LimitingParameter(zeta=0.1, eta=0.1),
                    rhs=ESLimitedLowOrderPos(low_order_surface_flux=LaxFriedrichsOnProjectedVal(),
                                             high_order_surface_flux=LaxFriedrichsOnProjectedVal()))
    exact = sedov_exact(param.equation.gamma)

    def initial_condition(param, x, y):
        return primitive_to_conservative(param.equation, exact(param.equation, x, y, 0.0))

    return param, initial_condition, periodic_bc, exact


def kpp_exact(equation=None, x=None, y=None, t=0.0):
    """exact_sol of examples/2D/KPP.jl:9-16 (the initial data): 7 pi / 2 in the unit disc,
    pi / 4 outside."""
    r2 = np.asarray(x) ** 2 + np.asarray(y) ** 2
    return np.where(r2 <= 1, 7 * np.pi / 2, np.pi / 4)


def kpp(N=3, Kx=64, Ky=64, T=1.0, rhs_limiter=None, reference_semantics=True, **kw):
    """examples/2D/KPP.jl:40-55: KPP{Dim2} on the periodic [-2, 2]^2, LGL nodes,
    ESLimitedLowOrderPos(LaxFriedrichsOnProjectedVal, LaxFriedrichsOnProjectedVal),
    SubcellLimiter(shockcapture=HennemannShockCapture()), zeta 0.1, eta 1.0, CFL 0.5,
    dt0 1e-3."""
    from dataclasses import replace

    from .types import HennemannShockCapture, KPP, LaxFriedrichsOnProjectedVal

    kw.setdefault("CFL", 0.5)
    kw.setdefault("dt0", 1e-3)
    if rhs_limiter is None:
        rhs_limiter = SubcellLimiter(shockcapture=HennemannShockCapture())
    param = default_param(N, (Kx, Ky), (-2.0, -2.0), (2.0, 2.0), T, rhs_limiter=rhs_limiter,
                          reference_semantics=reference_semantics, **kw)
    param = replace(param, equation=KPP(), limiting_param=LimitingParameter(zeta=0.1, eta=1.0),
                    rhs=ESLimitedLowOrderPos(low_order_surface_flux=LaxFriedrichsOnProjectedVal(),
                                             high_order_surface_flux=LaxFriedrichsOnProjectedVal()))

    def initial_condition(param, x, y):
        return kpp_exact(param.equation, x, y, 0.0)

    return param, initial_condition, periodic_bc, kpp_exact


def isentropic_vortex_exact(strength=8.5, x0=4.5, y0=5.0, ux=1.0, uy=0.0):
    """exact_sol of test/test_smoke.jl:6-20 with strength beta and advection (ux, uy)."""

    def exact_sol(equation, x, y, t):
        gamma = equation.gamma
        xs, ys = x - x0 - ux * t, y - y0 - uy * t
        r2 = xs**2 + ys**2
        u = ux - strength * np.exp(1 - r2) * ys / (2 * np.pi)
        v = uy + strength * np.exp(1 - r2) * xs / (2 * np.pi)
        rho = 1 - (1 / (8 * gamma * np.pi**2)) * (gamma - 1) / 2 * (strength * np.exp(1 - r2)) ** 2
        rho = rho ** (1 / (gamma - 1))
        p = rho**gamma
        return (rho, u, v, p)

    return exact_sol


def isentropic_vortex(N=3, Kx=5, Ky=5, T=0.02, strength=8.5, ux=1.0, uy=0.0, **kw):
    """test/test_smoke.jl: periodic [0,10]^2, vortex at (4.5, 5) advected by (ux, uy)."""
    kw.setdefault("CFL", 1.0)
    kw.setdefault("dt0", 1e-2)
    param = default_param(N, (Kx, Ky), (0.0, 0.0), (10.0, 10.0), T, **kw)
    exact = isentropic_vortex_exact(strength, 4.5, 5.0, ux, uy)
    t0 = param.timestepping_param.t0

    def initial_condition(param, x, y):
        return primitive_to_conservative(param.equation, exact(param.equation, x, y, t0))

    return param, initial_condition, periodic_bc, exact


def with_precision(param: Param, precision: str) -> Param:
    return replace(param, precision=precision)
