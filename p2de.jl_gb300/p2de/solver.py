"""initialize_DG / rhs! / SSP33! on top of libp2de_gpu.so.

Mirrors src/dg/init.jl:44-60 (initialize_DG), src/dg/rhs/rhs.jl:5-13 (rhs!) and
src/timestepping/SSPRK33.jl:1-62 (SSP33!). `!` is not allowed in Python names,
so rhs! and SSP33! are rhs_bang and SSP33_bang.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_int32, c_int64, c_void_p
from dataclasses import dataclass

import numpy as np

from . import abi
from .mesh import MeshData, uniform_mesh, uniform_mesh_1d
from .types import (
    BCData,
    DataHistory,
    ErrorData,
    ESLimitedLowOrderPos,
    EntropyStable,
    LaxFriedrichsOnNodalVal,
    LaxFriedrichsOnProjectedVal,
    GaussCollocation,
    LobattoCollocation,
    NodewiseScaledExtrapolation,
    LowOrderPositivity,
    NoEntropyProjectionLimiter,
    NoShockCapture,
    Param,
    PositivityAndCellEntropyBound,
    PositivityAndMinEntropyBound,
    PositivityAndRelaxedCellEntropyBound,
    PositivityAndRelaxedMinEntropyBound,
    PositivityBound,
    SubcellLimiter,
    TimeParam,
    TVDAndCellEntropyBound,
    TVDAndMinEntropyBound,
    TVDAndRelaxedCellEntropyBound,
    TVDAndRelaxedMinEntropyBound,
    TVDBound,
    HennemannShockCapture,
    ZhangShuLimiter,
    KPP,
    is_dim1,
    num_components,
)


class UnsupportedMethod(ValueError):
    pass


# SubcellLimiter bound types (Solver.jl:47-62) -> p2de_bound_type
BOUND_CODES = {
    PositivityBound: abi.BOUND_POSITIVITY,
    PositivityAndCellEntropyBound: abi.BOUND_POSITIVITY_AND_CELL_ENTROPY,
    TVDBound: abi.BOUND_TVD,
    TVDAndCellEntropyBound: abi.BOUND_TVD_AND_CELL_ENTROPY,
    PositivityAndMinEntropyBound: abi.BOUND_POSITIVITY_AND_MIN_ENTROPY,
    PositivityAndRelaxedMinEntropyBound: abi.BOUND_POSITIVITY_AND_RELAXED_MIN_ENTROPY,
    PositivityAndRelaxedCellEntropyBound: abi.BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY,
    TVDAndMinEntropyBound: abi.BOUND_TVD_AND_MIN_ENTROPY,
    TVDAndRelaxedMinEntropyBound: abi.BOUND_TVD_AND_RELAXED_MIN_ENTROPY,
    TVDAndRelaxedCellEntropyBound: abi.BOUND_TVD_AND_RELAXED_CELL_ENTROPY,
}


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64).ravel())


def _f64(a, shape=None) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        arr = arr.reshape(shape)
    return arr


@dataclass
class Descriptor:
    """The C descriptors of one solve plus the arrays they point into."""

    param: abi.P2deParam
    mesh: abi.P2deMesh
    keep: tuple
    N: int
    K: int
    dim1: bool = False

    @property
    def Nq(self) -> int:
        return self.N + 1 if self.dim1 else (self.N + 1) ** 2

    @property
    def Nfp(self) -> int:
        return 2 if self.dim1 else 4 * (self.N + 1)


def lower_param(param: Param, K: int) -> abi.P2deParam:
    """Maps the dispatch types of Param to the C enums, rejecting what is not built."""
    if isinstance(param.approximation_basis, LobattoCollocation):
        basis = abi.BASIS_LOBATTO
    elif isinstance(param.approximation_basis, GaussCollocation):
        basis = abi.BASIS_GAUSS
    else:
        raise UnsupportedMethod(f"basis {type(param.approximation_basis).__name__} is not built")
    if isinstance(param.entropyproj_limiter, NoEntropyProjectionLimiter):
        eproj = abi.ENTROPYPROJ_NONE
    elif isinstance(param.entropyproj_limiter, NodewiseScaledExtrapolation):
        eproj = abi.ENTROPYPROJ_NODEWISE_SCALED_EXTRAPOLATION
    else:
        raise UnsupportedMethod(f"entropy projection limiter {type(param.entropyproj_limiter).__name__} is not built")
    rhs = param.rhs
    if isinstance(rhs, ESLimitedLowOrderPos):
        rhs_type = abi.RHS_ES_LIMITED_LOW_ORDER_POS
        low, high = rhs.low_order_surface_flux, rhs.high_order_surface_flux
    elif isinstance(rhs, LowOrderPositivity):
        rhs_type = abi.RHS_LOW_ORDER_POSITIVITY
        low, high = rhs.surface_flux, LaxFriedrichsOnProjectedVal()
    elif isinstance(rhs, EntropyStable):
        rhs_type = abi.RHS_ENTROPY_STABLE
        low, high = LaxFriedrichsOnNodalVal(), rhs.surface_flux
    else:
        raise UnsupportedMethod(f"rhs type {type(rhs).__name__} is not built")
    if not isinstance(high, LaxFriedrichsOnProjectedVal):
        raise UnsupportedMethod("high-order surface flux: LaxFriedrichsOnProjectedVal")
    if isinstance(low, LaxFriedrichsOnNodalVal):
        low_code = abi.FLUX_LF_NODAL
    elif isinstance(low, LaxFriedrichsOnProjectedVal):
        low_code = abi.FLUX_LF_PROJECTED
    else:
        raise UnsupportedMethod("low-order surface flux: LaxFriedrichsOnNodalVal or LaxFriedrichsOnProjectedVal")
    kpp = isinstance(param.equation, KPP)
    lim = param.rhs_limiter
    bound = abi.BOUND_POSITIVITY
    limiter, beta = abi.LIMITER_SUBCELL, 0.0
    shock, sc_a, sc_c = 0, 0.0, 0.0
    if rhs_type == abi.RHS_ES_LIMITED_LOW_ORDER_POS:
        if isinstance(lim, ZhangShuLimiter):
            limiter = abi.LIMITER_ZHANG_SHU
        elif not isinstance(lim, SubcellLimiter):
            raise UnsupportedMethod("LimitedDG needs SubcellLimiter or ZhangShuLimiter")
        if isinstance(lim.shockcapture, HennemannShockCapture):
            shock, sc_a, sc_c = 1, float(lim.shockcapture.a), float(lim.shockcapture.c)
        elif not isinstance(lim.shockcapture, NoShockCapture):
            raise UnsupportedMethod(f"shock capture {type(lim.shockcapture).__name__} is not built")
        if isinstance(lim, SubcellLimiter):
            code = BOUND_CODES.get(type(lim.bound))
            if code is None:
                raise UnsupportedMethod(f"bound {type(lim.bound).__name__} is not built")
            bound = code
            beta = float(getattr(lim.bound, "beta", 0.0))
            if kpp and not isinstance(lim.bound, PositivityBound):
                raise UnsupportedMethod("KPP: the subcell limiter reads no bound; use PositivityBound")
    if kpp and basis != abi.BASIS_LOBATTO:
        raise UnsupportedMethod("KPP on LGL nodes only")
    if param.precision not in abi.PRECISIONS:
        raise UnsupportedMethod("precision must be one of " + ", ".join(abi.PRECISIONS))
    gc, ts, lp = param.global_constants, param.timestepping_param, param.limiting_param
    return abi.P2deParam(
        N=param.N,
        K=K,
        gamma=getattr(param.equation, "gamma", 1.4),
        POSTOL=gc.POSTOL,
        ZEROTOL=gc.ZEROTOL,
        zeta=lp.zeta,
        eta=lp.eta,
        CFL=ts.CFL,
        dt0=ts.dt0,
        t0=ts.t0,
        T=ts.T,
        rhs_type=rhs_type,
        bound_type=bound,
        low_order_surface_flux=low_code,
        high_order_surface_flux=abi.FLUX_LF_PROJECTED,
        shock_capture=shock,
        shock_capture_a=sc_a,
        shock_capture_c=sc_c,
        rhs_limiter=limiter,
        bound_beta=beta,
        approximation_basis=basis,
        entropyproj_limiter=eproj,
        equation=abi.EQUATION_KPP if kpp else (abi.EQUATION_COMPRESSIBLE_EULER_1D if is_dim1(param.equation)
                                               else abi.EQUATION_COMPRESSIBLE_EULER),
        reference_semantics=1 if param.reference_semantics else 0,
        precision=abi.PRECISIONS[param.precision],
    )


def mesh_for(param: Param) -> MeshData:
    """The uniform mesh of initialize_uniform_mesh_data (init.jl:241-252) with the nodes
    of param's basis."""
    basis = "gauss" if isinstance(param.approximation_basis, GaussCollocation) else "lobatto"
    if is_dim1(param.equation):  # initialize_uniform_mesh_data(::Line) (init.jl:230-239)
        return uniform_mesh_1d(param.N, int(param.K), float(param.xL), float(param.xR), basis=basis)
    return uniform_mesh(param.N, param.K[0], param.K[1], param.xL, param.xR, basis=basis)


def make_descriptor(param: Param, md: MeshData, bc: BCData) -> Descriptor:
    K = md.num_elements
    geom = _f64(md.geom)
    mapP = _i64(bc.mapP)
    mapI, mapO, mapW, mapS = _i64(bc.mapI), _i64(bc.mapO), _i64(bc.mapW), _i64(bc.mapS)
    dim1 = is_dim1(param.equation)
    nc = 3 if dim1 else 4
    Ival = _f64(bc.Ival if len(bc.Ival) else np.zeros((0, nc))).reshape(-1, nc)
    xyS = _f64(bc.xyS if len(bc.xyS) else np.zeros((0, 2))).reshape(-1, 2)
    if mapP.size != K * (2 if dim1 else 4 * (param.N + 1)):
        raise ValueError("mapP has the wrong size")
    m = abi.P2deMesh()
    m.geom = abi.dptr(geom)
    m.mapP = abi.iptr(mapP)
    m.mapI, m.nI = abi.iptr(mapI), mapI.size
    m.Ival = abi.dptr(Ival)
    m.mapO, m.nO = abi.iptr(mapO), mapO.size
    m.mapW, m.nW = abi.iptr(mapW), mapW.size
    m.mapS, m.nS = abi.iptr(mapS), mapS.size
    m.xyS = abi.dptr(xyS)
    m.shock_x0 = bc.shock_x0
    m.shock_inv_slope = bc.shock_inv_slope
    m.shock_speed = bc.shock_speed
    for c in range(4):
        m.shock_post[c] = bc.shock_post[c]
        m.shock_pre[c] = bc.shock_pre[c]
    p = lower_param(param, K)
    return Descriptor(p, m, (geom, mapP, mapI, mapO, mapW, mapS, Ival, xyS), param.N, K, dim1)


def evaluate_initial_condition(param: Param, md: MeshData, initial_condition) -> np.ndarray:
    """init_U! (init.jl:342-361): Uq[i,k] = initial_condition(param, x, y), vectorised.
    Returns (K, Nq, Nc) float64 (Julia's Uq memory layout); on a Line initial_condition(param,
    x) (set_initial_condition!(::Dim1), init.jl:352-355)."""
    u = initial_condition(param, md.x) if md.dim1 else initial_condition(param, md.x, md.y)
    if isinstance(u, (tuple, list)):
        u = np.stack([np.broadcast_to(np.asarray(c, dtype=np.float64), md.x.shape) for c in u], axis=-1)
    u = np.ascontiguousarray(np.asarray(u, dtype=np.float64))
    nc = num_components(param.equation)
    if nc == 1 and u.shape == md.x.shape:
        u = u[..., None]
    if u.shape != md.x.shape + (nc,):
        raise ValueError(f"initial condition returned shape {u.shape}, expected {md.x.shape + (nc,)}")
    return u


class Solver:
    """Solver (Solver.jl:220-225) holding the GPU handle."""

    def __init__(self, param: Param, md: MeshData, desc: Descriptor, device: int = 0):
        self.param = param
        self.md = md
        self.desc = desc
        self.lib = abi.load_library()
        h = c_void_p()
        st = self.lib.p2de_initialize_DG(byref(desc.param), byref(desc.mesh), device, byref(h))
        abi.check(self.lib, st, None)
        self.handle = h
        self.K = desc.K
        self.N = param.N
        self.N1D = param.N + 1
        self.Nq = desc.Nq
        self.Nfp = desc.Nfp

    def close(self):
        if getattr(self, "handle", None):
            self.lib.p2de_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        abi.check(self.lib, st, self.handle)

    def field_count(self, field: int) -> int:
        c = c_int64()
        self._check(self.lib.p2de_solver_field_count(self.handle, field, byref(c)))
        return c.value

    def get_field(self, field: int, nstage: int = 1) -> np.ndarray:
        out = np.empty(self.field_count(field), dtype=np.float64)
        self._check(self.lib.p2de_get_field(self.handle, field, nstage, abi.dptr(out)))
        return out

    def set_Uq(self, Uq: np.ndarray) -> None:
        U = np.ascontiguousarray(Uq, dtype=np.float64)
        if U.size != self.field_count(abi.FIELD_UQ):
            raise ValueError("Uq has the wrong size")
        self._check(self.lib.p2de_set_Uq(self.handle, abi.dptr(U)))

    def launch_count(self) -> int:
        c = c_int64()
        self._check(self.lib.p2de_launch_count(self.handle, byref(c)))
        return c.value

    def elements_per_block(self) -> tuple[int, int]:
        """(current, largest) elements per thread block of the stage kernels."""
        e, m = c_int32(), c_int32()
        self._check(self.lib.p2de_get_elements_per_block(self.handle, byref(e), byref(m)))
        return e.value, m.value

    def set_elements_per_block(self, epb: int) -> None:
        self._check(self.lib.p2de_set_elements_per_block(self.handle, int(epb)))

    def layout(self) -> int:
        """Thread layout (abi.LAYOUT_*): of the high-order pair phases of a 2D solve (FLAT or
        LINES_PER_WARP), of the Line kernels of a 1D solve (FLAT or TEAM)."""
        v = c_int32()
        self._check(self.lib.p2de_get_layout(self.handle, byref(v)))
        return v.value

    def set_layout(self, layout: int) -> None:
        self._check(self.lib.p2de_set_layout(self.handle, int(layout)))

    def threads_per_block(self) -> int:
        v = c_int32()
        self._check(self.lib.p2de_get_threads_per_block(self.handle, byref(v)))
        return v.value

    def set_threads_per_block(self, threads: int) -> None:
        self._check(self.lib.p2de_set_threads_per_block(self.handle, int(threads)))

    def autotune(self) -> tuple[int, float]:
        """Keeps the fastest elements-per-block, thread layout and block size for stage kernel A;
        returns the elements per block with its ms (layout() gives the layout kept)."""
        e, ms = c_int32(), c_double()
        self._check(self.lib.p2de_autotune(self.handle, byref(e), byref(ms)))
        return e.value, ms.value


class State:
    """State (State.jl:258-261): the preallocated arrays live on the device."""

    def __init__(self, solver: Solver):
        self._s = solver

    @property
    def Uq(self) -> np.ndarray:
        """(K, Nq, Nc): Nc = 4, 1 (KPP) or 3 (CompressibleEulerIdealGas{Dim1})."""
        return self._s.get_field(abi.FIELD_UQ).reshape(self._s.K, self._s.Nq, -1)

    @Uq.setter
    def Uq(self, value):
        self._s.set_Uq(value)

    def field(self, field: int, nstage: int = 1) -> np.ndarray:
        return self._s.get_field(field, nstage)

    @property
    def rhsU(self):
        return self.field(abi.FIELD_RHSU).reshape(self._s.K, self._s.Nq, -1)

    @property
    def rhsL(self):
        return self.field(abi.FIELD_RHSL).reshape(self._s.K, self._s.Nq, -1)

    @property
    def rhsH(self):
        return self.field(abi.FIELD_RHSH).reshape(self._s.K, self._s.Nq, -1)

    def L_local(self, nstage: int) -> np.ndarray:
        """L_local[:, :, :, nstage] as (K, Nd, Nq + N1D)."""
        nd = 1 if self._s.desc.dim1 else 2
        return self.field(abi.FIELD_L_LOCAL, nstage).reshape(self._s.K, nd, self._s.Nq + self._s.N1D)


@dataclass
class StateParam:
    bcdata: BCData


def initialize_DG(param: Param, initial_condition, initial_boundary_conditions, device: int = 0):
    """initialize_DG(param, initial_condition, initial_boundary_conditions)
    (init.jl:44-60) -> (solver, state, state_param)."""
    md = mesh_for(param)
    bcdata = initial_boundary_conditions(param, md)
    desc = make_descriptor(param, md, bcdata)
    solver = Solver(param, md, desc, device)
    state = State(solver)
    solver.set_Uq(evaluate_initial_condition(param, md, initial_condition))
    return solver, state, StateParam(bcdata)


@dataclass
class Preallocation:
    """The members of Preallocation (State.jl:1-26) that SSP33! and its callers read and
    write, as host arrays: Uq, rhsU, resW, resZ (K, Nq, Nc) and L_local (Ns, K, Nd, Nq+N1D)."""

    Uq: np.ndarray
    rhsU: np.ndarray
    resW: np.ndarray
    resZ: np.ndarray
    L_local: np.ndarray


class HostState:
    """State (State.jl:258-261) holding host arrays, as the reference's does: the caller
    mutates preallocation.Uq between right-hand-side evaluations (SSP33!, SSPRK33.jl:30-39),
    and rhs_bang uploads Uq before and downloads rhsU and the stage's L_local after the
    device evaluation."""

    def __init__(self, solver, Uq: np.ndarray):
        """solver: a Solver, or anything with param, K, Nq, N1D and desc (Descriptor)."""
        nc = num_components(solver.param.equation)
        U = np.array(Uq, dtype=np.float64).reshape(solver.K, solver.Nq, nc)
        nd = 1 if solver.desc.dim1 else 2
        self.preallocation = Preallocation(
            Uq=U, rhsU=np.zeros_like(U), resW=np.zeros_like(U), resZ=np.zeros_like(U),
            L_local=np.ones((3, solver.K, nd, solver.Nq + solver.N1D)))


def rhs_bang(state, solver: Solver, state_param: StateParam, time_param: TimeParam) -> float:
    """rhs!(state, solver, state_param, time_param) (rhs.jl:5-13): fills rhsU, returns dt.

    With a HostState, Uq is read from state.preallocation.Uq and rhsU (and, under the
    subcell limiter, L_local[:, :, :, nstage]) written back to it, so host code that changes
    Uq between stages sees the reference's behaviour. With a device-resident State (or
    None) the device Uq is used as it is."""
    host = isinstance(state, HostState)
    if host:
        solver.set_Uq(state.preallocation.Uq)
    out = c_double()
    solver._check(solver.lib.p2de_rhs(solver.handle, time_param.t, time_param.dt, time_param.nstage, byref(out)))
    if host:
        pre = state.preallocation
        pre.rhsU[...] = solver.get_field(abi.FIELD_RHSU).reshape(pre.rhsU.shape)
        lim = solver.param.rhs_limiter
        if isinstance(solver.param.rhs, ESLimitedLowOrderPos) and isinstance(lim, SubcellLimiter):
            s = time_param.nstage - 1
            pre.L_local[s] = solver.get_field(abi.FIELD_L_LOCAL, time_param.nstage).reshape(pre.L_local[s].shape)
    return out.value


def SSP33_host_loop(state: HostState, solver, state_param: StateParam, nsteps: int | None = None, rhs=None,
                    t_start: float | None = None):
    """The time loop of SSP33! (SSPRK33.jl:25-41) written over host arrays, calling rhs!
    (rhs_bang unless `rhs` is given) three times per step exactly as the reference does:
    resW = Uq; dt = rhs!(stage 1); Uq = resW + dt rhsU; rhs!(stage 2); resZ = Uq + dt rhsU;
    Uq = 3/4 resW + 1/4 resZ; rhs!(stage 3); resZ = Uq + dt rhsU; Uq = 1/3 resW + 2/3 resZ.
    Starts at t_start (default t0) and stops at T or after nsteps steps; returns
    (t, dt history)."""
    rhs_bang_ = rhs if rhs is not None else rhs_bang
    ts = solver.param.timestepping_param
    pre = state.preallocation
    t = ts.t0 if t_start is None else t_start
    dthist = []
    while t < ts.T and (nsteps is None or len(dthist) < nsteps):
        dt = min(ts.CFL * ts.dt0, ts.T - t)
        pre.resW[...] = pre.Uq
        dt = rhs_bang_(state, solver, state_param, TimeParam(t, dt, 1))
        pre.Uq[...] = pre.resW + dt * pre.rhsU
        rhs_bang_(state, solver, state_param, TimeParam(t, dt, 2))
        pre.resZ[...] = pre.Uq + dt * pre.rhsU
        pre.Uq[...] = 3 / 4 * pre.resW + 1 / 4 * pre.resZ
        rhs_bang_(state, solver, state_param, TimeParam(t, dt, 3))
        pre.resZ[...] = pre.Uq + dt * pre.rhsU
        pre.Uq[...] = 1 / 3 * pre.resW + 2 / 3 * pre.resZ
        t = t + dt
        dthist.append(dt)
    return t, dthist


def ssp33_step(solver: Solver, t: float) -> tuple[float, float]:
    """One pass of the SSP33! loop body (SSPRK33.jl:125-139); returns (t_new, dt)."""
    tt, dt = c_double(t), c_double()
    solver._check(solver.lib.p2de_ssp33_step(solver.handle, byref(tt), byref(dt)))
    return tt.value, dt.value


def ssp33(solver: Solver) -> tuple[float, int, float]:
    """The whole SSP33! time loop (SSPRK33.jl:1-62) on the device without snapshots;
    returns (t, steps, last dt)."""
    t, n, dt = c_double(), c_int64(), c_double()
    solver._check(solver.lib.p2de_ssp33(solver.handle, byref(t), byref(n), byref(dt)))
    return t.value, n.value, dt.value


def SSP33_bang(state: State, solver: Solver, state_param: StateParam, snapshots: bool = True) -> DataHistory:
    """SSP33!(state, solver, state_param) (SSPRK33.jl:1-62). Steps on the device in
    CUDA-graph chunks up to each snapshot index (mod(i, output_interval) == 0) and
    records the final state, as the reference does at |t - T| < 1e-10."""
    ts = solver.param.timestepping_param
    interval = max(1, solver.param.postprocessing_param.output_interval)
    t = ts.t0
    i = 1
    hist = DataHistory([], [], [], [], [])
    while t < ts.T:
        nxt = interval - (i % interval) if snapshots else 1 << 20
        tt, done = c_double(t), c_int64()
        solver._check(solver.lib.p2de_ssp33_advance(solver.handle, nxt, byref(tt), byref(done)))
        if done.value == 0:
            break
        t = tt.value
        i += done.value
        if snapshots and (i % interval == 0 or abs(t - ts.T) < 1e-10):
            hist.thist.append(t)
            hist.Uhist.append(state.Uq.copy())
            hist.Lhist.append(state.L_local(3).copy())
    return hist


def check_conservation(state: State, solver: Solver) -> float:
    """check_conservation (src/dg/utils.jl:1-12): sum of J*wq*Uq over nodes and
    components, reduced on the device."""
    total = c_double()
    solver._check(solver.lib.p2de_check_conservation(solver.handle, None, byref(total)))
    return total.value


def conservation_totals(solver: Solver) -> np.ndarray:
    """The four component totals of check_conservation."""
    out = np.zeros(4)
    solver._check(solver.lib.p2de_check_conservation(solver.handle, abi.dptr(out), None))
    return out


def exact_nodal_values(solver: Solver, exact_sol, t: float) -> np.ndarray:
    """exact_solution(::CompressibleIdealGas{Dim2}, ...) (src/dg/postprocess.jl:54-59) at
    every node: conservative values in the layout of Uq."""
    from .problems import primitive_to_conservative

    if solver.md.dim1:  # exact_solution(::CompressibleIdealGas{Dim1}) (postprocess.jl:48-52)
        prim = exact_sol(solver.param.equation, solver.md.x, t)
    else:
        prim = exact_sol(solver.param.equation, solver.md.x, solver.md.y, t)
    return np.ascontiguousarray(primitive_to_conservative(solver.param.equation, prim), dtype=np.float64)


def calculate_error(state: State, solver: Solver, exact_sol) -> ErrorData:
    """calculate_error (src/dg/postprocess.jl:1-46): relative L1/L2/Linf summed over
    components, against exact_sol(equation, x, y, T) returning (rho, u, v, p); the
    norms are reduced on the device."""
    Ue = exact_nodal_values(solver, exact_sol, solver.param.timestepping_param.T)
    out = np.zeros(3)
    solver._check(solver.lib.p2de_calculate_error(solver.handle, abi.dptr(Ue), abi.dptr(out)))
    return ErrorData(float(out[0]), float(out[1]), float(out[2]))
