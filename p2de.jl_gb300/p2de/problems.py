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
    vectorised: (rho, u, v, p) arrays -> (..., 4); (rho, u, p) -> (..., 3) on a Line."""
    gamma = equation.gamma
    if len(prim) == 3:  # primitive_to_conservative(::CompressibleIdealGas{Dim1}) (:1-7)
        rho, u, p = np.broadcast_arrays(*(np.asarray(a, dtype=np.float64) for a in prim))
        return np.stack([rho, rho * u, p / (gamma - 1) + 0.5 * rho * u**2], axis=-1)
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


def sedov_lgl(N=3, Kx=16, Ky=16, T=0.05, r_ini=0.3, **kw):
    """The Sedov initial data of examples/2D/sedov.jl:9-20 (rho 1 at rest, pressure
    (gamma - 1) / (pi r_ini^2) inside r < r_ini and 1e-5 outside) on the periodic
    [-1.5, 1.5]^2 with LGL nodes and the default method of default_param (subcell limiter),
    r_ini wide enough to cover a few elements: a blast that keeps the limiter busy."""
    param = default_param(N, (Kx, Ky), (-1.5, -1.5), (1.5, 1.5), T, **kw)
    exact = sedov_exact(param.equation.gamma, r_ini=r_ini)

    def initial_condition(param, x, y):
        return primitive_to_conservative(param.equation, exact(param.equation, x, y, 0.0))

    return param, initial_condition, periodic_bc


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


# --- CompressibleEulerIdealGas{Dim1} --------------------------------------------------
# The reference's Dim1 path raises before its first RHS (Bx(::Dim1) calls
# reference_to_physical with its arguments in the wrong order, rhs_utils.jl:18), so these
# problems run with reference_semantics=False: the Dim1 methods with their evident meaning.
def line_param(N, K, xL, xR, T, gamma=1.4, CFL=0.5, dt0=None, t0=0.0, zeta=0.1, eta=0.5, rhs_limiter=None,
               approximation_basis=None, entropyproj_limiter=None, rhs=None, **kw):
    """Param of a CompressibleEulerIdealGas{Dim1} solve on [xL, xR] with K elements."""
    from .types import Dim1, PositivityBound

    if rhs_limiter is None:
        rhs_limiter = SubcellLimiter(bound=PositivityBound())
    kw.pop("reference_semantics", None)
    p = default_param(N, (K, 1), (xL, 0.0), (xR, 0.0), T, CFL=CFL, dt0=dt0, rhs_limiter=rhs_limiter,
                      approximation_basis=approximation_basis, entropyproj_limiter=entropyproj_limiter,
                      reference_semantics=False, **kw)
    return replace(p, K=int(K), xL=float(xL), xR=float(xR), equation=CompressibleEulerIdealGas(gamma, Dim1),
                   limiting_param=LimitingParameter(zeta=zeta, eta=eta),
                   timestepping_param=TimesteppingParameter(T=T, CFL=CFL, dt0=T if dt0 is None else dt0, t0=t0),
                   rhs=rhs if rhs is not None else ESLimitedLowOrderPos())


def inflow_outflow_1d(state_left):
    """initial_boundary_conditions of examples/1D/shu-osher.jl:16-32: mapI = [1] with the
    conservative state_left, mapO = [2K], mapP of the Line mesh."""

    def bc(param, md: MeshData) -> BCData:
        K = md.num_elements
        return BCData(mapP=md.mapP, mapI=np.array([1]), mapO=np.array([2 * K]),
                      Ival=np.asarray(state_left, dtype=np.float64).reshape(1, 3))

    return bc


def shu_osher_exact(equation=None, x=None, t=0.0):
    """exact_sol of examples/1D/shu-osher.jl:8-14 (the initial data)."""
    x = np.asarray(x, dtype=np.float64)
    left = x < -4.0
    rho = np.where(left, 3.857143, 1 + 0.2 * np.sin(5 * x))
    u = np.where(left, 2.629369, 0.0)
    p = np.where(left, 10.3333, 1.0)
    return rho, u, p


def shu_osher(N=3, K=64, T=1.8, **kw):
    """examples/1D/shu-osher.jl:44-56: [-5, 5], gamma 1.4, CFL 0.5, dt0 1e-4, zeta 0.1,
    eta 1.0, GaussCollocation with NodewiseScaledExtrapolation, ESLimitedLowOrderPos(
    LaxFriedrichsOnNodalVal, LaxFriedrichsOnProjectedVal), SubcellLimiter(PositivityBound)."""
    from .types import GaussCollocation, NodewiseScaledExtrapolation

    kw.setdefault("dt0", 1e-4)
    kw.setdefault("eta", 1.0)
    kw.setdefault("approximation_basis", GaussCollocation())
    kw.setdefault("entropyproj_limiter", NodewiseScaledExtrapolation())
    param = line_param(N, K, -5.0, 5.0, T, **kw)
    eq = param.equation

    def initial_condition(param, x):
        return primitive_to_conservative(param.equation, shu_osher_exact(param.equation, x, 0.0))

    left = primitive_to_conservative(eq, (3.857143, 2.629369, 10.3333))
    return param, initial_condition, inflow_outflow_1d(left), shu_osher_exact


def leblanc_exact(equation, x, t):
    """exact_sol of examples/convergence/leblanc-convergence.jl:9-40: the Leblanc shock tube
    (rho 1 | 1e-3, p (gamma-1) 1e-1 | (gamma-1) 1e-10, interface at x = 0.33)."""
    gamma = equation.gamma
    x = np.asarray(x, dtype=np.float64)
    rhoL, rhoR, pL, pR = 1.0, 1e-3, (gamma - 1) * 1e-1, (gamma - 1) * 1e-10
    if t == 0:
        left = x < 0.33
        return np.where(left, rhoL, rhoR), np.zeros_like(x), np.where(left, pL, pR)
    xi = (x - 0.33) / t
    rhoLstar, rhoRstar = 5.4079335349316249e-2, 3.9999980604299963e-3
    vstar, pstar = 0.62183867139173454, 0.51557792765096996e-3
    lambda1, lambda3 = 0.49578489518897934, 0.82911836253346982
    fan = (xi > -1 / 3) & (xi <= lambda1)
    rho = np.select([xi <= -1 / 3, fan, xi <= vstar, xi <= lambda3], [rhoL, (0.75 - 0.75 * xi) ** 3, rhoLstar, rhoRstar], rhoR)
    u = np.select([xi <= -1 / 3, fan, xi <= lambda3], [0.0, 0.75 * (1 / 3 + xi), vstar], 0.0)
    p = np.select([xi <= -1 / 3, fan, xi <= lambda3], [pL, 1 / 15 * (0.75 - 0.75 * xi) ** 5, pstar], pR)
    return rho, u, p


def leblanc(N=2, K=50, T=2 / 3, **kw):
    """examples/convergence/leblanc-convergence.jl:75-89: [0, 1], gamma 5/3, CFL 0.5, dt0 1e-3,
    t0 0.01 (the initial data is the exact solution there), zeta 0.1, eta 0.1; inflow at the
    left end, outflow at the right. The limiter and basis come from kw (default
    SubcellLimiter(PositivityBound) on LGL nodes)."""
    kw.setdefault("dt0", 1e-3)
    kw.setdefault("eta", 0.1)
    kw.setdefault("t0", 0.01)
    param = line_param(N, K, 0.0, 1.0, T, gamma=5 / 3, **kw)
    eq = param.equation

    def initial_condition(param, x):
        t0 = param.timestepping_param.t0
        return primitive_to_conservative(param.equation, leblanc_exact(param.equation, x, t0))

    left = primitive_to_conservative(eq, (1.0, 0.0, (eq.gamma - 1) * 1e-1))
    return param, initial_condition, inflow_outflow_1d(left), leblanc_exact


def density_wave_1d_exact(equation=None, x=None, t=0.0, amp=0.2, u=1.0, p=1.0):
    """A smooth periodic density wave on [0, 1]: rho = 1 + amp sin(2 pi (x - u t)), u, p
    constant (an exact Euler solution)."""
    x = np.asarray(x, dtype=np.float64)
    return 1.0 + amp * np.sin(2 * np.pi * (x - u * t)), np.full_like(x, u), np.full_like(x, p)


def density_wave_1d(N=3, K=16, T=0.1, **kw):
    """The periodic density wave on [0, 1] (a smooth test of the Line path)."""

    param = line_param(N, K, 0.0, 1.0, T, **kw)

    def initial_condition(param, x):
        return primitive_to_conservative(param.equation, density_wave_1d_exact(param.equation, x, 0.0))

    def bc(param, md):
        from .mesh import uniform_mesh_1d
        basis = "gauss" if type(param.approximation_basis).__name__ == "GaussCollocation" else "lobatto"
        return BCData(mapP=uniform_mesh_1d(param.N, md.num_elements, md.xL[0], md.xR[0], basis, periodic=True).mapP)

    return param, initial_condition, bc, density_wave_1d_exact
