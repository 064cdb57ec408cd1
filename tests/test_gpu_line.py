"""GPU parity of CompressibleEulerIdealGas{Dim1} (the Line path) against the FP64 oracle.

The reference's own Dim1 path raises before its first RHS (Bx(::Dim1) passes its arguments
to reference_to_physical in the wrong order, rhs_utils.jl:18), so both sides run the Dim1
methods with their evident meaning (reference_semantics = False): the RHS of rhs.jl:183-213
on LGL and Gauss nodes (NodewiseScaledExtrapolation), the subcell limiter's Dim1 methods
(subcell.jl:144-246, 405-415, 468-628, 826-892) for every bound, Zhang-Shu, Hennemann shock
capture, periodic / inflow / outflow faces, and the examples' configurations
(examples/1D/shu-osher.jl, examples/convergence/leblanc-convergence.jl).

Both sides evaluate a*b+c as two rounded operations in the same order (the Line kernels are
compiled with -fmad=false), so single RHS evaluations agree to the last bits of log, exp and
pow, and runs to where a limiter decision turns on those bits.
"""
import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.types import (
    EntropyStable,
    ESLimitedLowOrderPos,
    GaussCollocation,
    HennemannShockCapture,
    LaxFriedrichsOnProjectedVal,
    LobattoCollocation,
    LowOrderPositivity,
    NodewiseScaledExtrapolation,
    NoEntropyProjectionLimiter,
    PositivityAndCellEntropyBound,
    PositivityAndMinEntropyBound,
    PositivityAndRelaxedCellEntropyBound,
    PositivityAndRelaxedMinEntropyBound,
    PositivityBound,
    SubcellLimiter,
    TVDAndCellEntropyBound,
    TVDAndMinEntropyBound,
    TVDBound,
    ZhangShuLimiter,
)

from conftest import relerr
from helpers import setup
from test_gpu_parity import TOL, gpu_for, oracle_for

pytestmark = pytest.mark.gpu

TOL_RUN = 1e-9
# The smooth density wave is ill-conditioned in the reference's own arithmetic: its node
# pairs put the log mean (compressible_Navier_Stokes.jl:307-321) just past the 1e-4
# threshold of its series, where -da / (log aL - log aR) magnifies one ulp of a log by
# 1e4. Perturbing the state by two ulps moves the oracle's own rhsU by up to 2.4e-11 (LGL)
# and 9.3e-11 (Gauss); Leblanc's and Shu-Osher's states move it by at most 2e-14.
TOL_WAVE = 1e-9

LIMITERS = {
    "pos": SubcellLimiter(bound=PositivityBound()),
    "cell": SubcellLimiter(bound=PositivityAndCellEntropyBound()),
    "relaxed-cell": SubcellLimiter(bound=PositivityAndRelaxedCellEntropyBound(beta=0.5)),
    "minent": SubcellLimiter(bound=PositivityAndMinEntropyBound()),
    "relaxed-minent": SubcellLimiter(bound=PositivityAndRelaxedMinEntropyBound()),
    "tvd": SubcellLimiter(bound=TVDBound()),
    "tvd-cell": SubcellLimiter(bound=TVDAndCellEntropyBound()),
    "tvd-minent": SubcellLimiter(bound=TVDAndMinEntropyBound()),
    "pos+hennemann": SubcellLimiter(bound=PositivityBound(), shockcapture=HennemannShockCapture()),
    "zhang-shu": ZhangShuLimiter(),
    "zhang-shu+hennemann": ZhangShuLimiter(shockcapture=HennemannShockCapture()),
}
CELL = ("cell", "relaxed-cell", "tvd-cell")


def basis_kw(basis):
    if basis == "gauss":
        return dict(approximation_basis=GaussCollocation(), entropyproj_limiter=NodewiseScaledExtrapolation())
    return dict(approximation_basis=LobattoCollocation(), entropyproj_limiter=NoEntropyProjectionLimiter())


def compare_line_rhs(param, md, desc, U0, t, dt, nstage, tol=TOL):
    o = oracle_for(desc, U0)
    g = gpu_for(param, md, desc, U0)
    dto = o.rhs(t, dt, nstage)
    dtg = S.rhs_bang(None, g, None, p2de.TimeParam(t, dt, nstage))
    assert abs(dtg - dto) <= 1e-13 * abs(dto), (dtg, dto)
    fields = [abi.FIELD_RHSL, abi.FIELD_RHSH, abi.FIELD_BF_L, abi.FIELD_BF_H, abi.FIELD_RHSU]
    if not isinstance(param.rhs, ESLimitedLowOrderPos):
        fields = [abi.FIELD_RHSU]
    for f in fields:
        a, b = g.get_field(f), o.get_field(f)
        assert a.size == b.size == g.field_count(f)
        assert relerr(a, b, floor=1e-300) <= tol, (f, relerr(a, b, floor=1e-300))
    th_g, th_o = g.get_field(abi.FIELD_THETA_LOCAL, nstage), o.get_field(abi.FIELD_THETA_LOCAL, nstage)
    np.testing.assert_allclose(th_g, th_o, rtol=0, atol=1e-15)
    lim = param.rhs_limiter
    if isinstance(param.rhs, ESLimitedLowOrderPos) and isinstance(lim, SubcellLimiter):
        n1 = param.N + 1
        Lg = g.get_field(abi.FIELD_L_LOCAL, nstage).reshape(desc.K, 2 * n1)[:, : n1 + 1]
        Lo = o.get_field(abi.FIELD_L_LOCAL, nstage).reshape(desc.K, 2 * n1)[:, : n1 + 1]
        assert np.all((Lg >= 0) & (Lg <= 1))
        # A factor is a decision when the subcell flux difference it limits is at the
        # rounding level (e.g. a TVD bound met with equality at a smooth extremum): one ulp
        # of the state flips it between 0 and 1 there, while its product with that
        # difference (rhsU, compared above) stays put. The factors that move when the
        # oracle's own input moves by two ulps are left out; the rest must agree.
        unstable = np.zeros(Lo.shape, dtype=bool)
        rng = np.random.default_rng(1)
        for _ in range(4):
            o.set_Uq(U0 * (1 + 2.2e-16 * rng.integers(-2, 3, np.shape(U0))))
            o.rhs(t, dt, nstage)
            Lp = o.get_field(abi.FIELD_L_LOCAL, nstage).reshape(desc.K, 2 * n1)[:, : n1 + 1]
            unstable |= np.abs(Lp - Lo) > max(tol, 1e-12)
        # (TVD bounds in Leblanc's flat states are met with equality in about one factor in
        # eight; the smooth wave has two such faces in sixty)
        assert unstable.sum() <= 0.5 * unstable.size
        np.testing.assert_allclose(Lg[~unstable], Lo[~unstable], rtol=0, atol=max(tol, 1e-12))
    if isinstance(lim, ZhangShuLimiter):
        np.testing.assert_allclose(g.get_field(abi.FIELD_L, nstage), o.get_field(abi.FIELD_L, nstage),
                                   atol=max(tol, 1e-12))
    g.close()
    o.close()


@pytest.mark.parametrize("basis", ["lobatto", "gauss"])
@pytest.mark.parametrize("limiter", list(LIMITERS))
@pytest.mark.parametrize("problem", ["density-wave", "leblanc"])
def test_line_rhs(basis, limiter, problem):
    if basis == "gauss" and limiter in CELL:
        pytest.skip("no cell-entropy bound on Gauss nodes in 1D (no Dim1 interface method)")
    kw = dict(rhs_limiter=LIMITERS[limiter], **basis_kw(basis))
    if problem == "density-wave":
        param, md, bc, desc, U0 = setup(problems.density_wave_1d, N=3, K=12, T=0.1, **kw)
        t0, tol = 0.0, TOL_WAVE
    else:
        param, md, bc, desc, U0 = setup(problems.leblanc, N=2, K=40, **kw)
        t0, tol = param.timestepping_param.t0, TOL
    for nstage in (1, 2):
        compare_line_rhs(param, md, desc, U0, t0, 1e-3, nstage, tol=tol)


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("basis", ["lobatto", "gauss"])
def test_line_rhs_degrees(N, basis):
    param, md, bc, desc, U0 = setup(problems.shu_osher, N=N, K=24, **basis_kw(basis))
    compare_line_rhs(param, md, desc, U0, 0.0, 1e-4, 1)


@pytest.mark.parametrize("rhs", ["low", "es", "lfproj"])
@pytest.mark.parametrize("basis", ["lobatto", "gauss"])
def test_line_rhs_types(rhs, basis):
    r = {"low": LowOrderPositivity(), "es": EntropyStable(),
         "lfproj": ESLimitedLowOrderPos(low_order_surface_flux=LaxFriedrichsOnProjectedVal())}[rhs]
    param, md, bc, desc, U0 = setup(problems.leblanc, N=3, K=30, rhs=r, **basis_kw(basis))
    compare_line_rhs(param, md, desc, U0, param.timestepping_param.t0, 1e-3, 1)


@pytest.mark.parametrize("limiter", ["pos", "minent", "tvd", "cell", "zhang-shu+hennemann"])
@pytest.mark.parametrize("basis", ["lobatto", "gauss"])
def test_line_steps(limiter, basis):
    if basis == "gauss" and limiter in CELL:
        pytest.skip("no cell-entropy bound on Gauss nodes in 1D")
    param, md, bc, desc, U0 = setup(problems.leblanc, N=2, K=50, T=0.05, rhs_limiter=LIMITERS[limiter],
                                    **basis_kw(basis))
    o = oracle_for(desc, U0)
    g = gpu_for(param, md, desc, U0)
    to = tg = param.timestepping_param.t0
    for _ in range(20):
        to, dto = o.step(to)
        tg, dtg = S.ssp33_step(g, tg)
        assert abs(dtg - dto) <= 1e-12 * dto
    assert relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)) <= TOL_RUN
    U = g.get_field(abi.FIELD_UQ).reshape(-1, 3)
    assert U[:, 0].min() > 0 and (U[:, 2] - 0.5 * U[:, 1] ** 2 / U[:, 0]).min() > 0
    g.close()
    o.close()


@pytest.mark.parametrize("basis", ["lobatto", "gauss"])
def test_line_periodic_conservation(basis):
    param, md, bc, desc, U0 = setup(problems.density_wave_1d, N=4, K=16, T=0.05,
                                    rhs_limiter=LIMITERS["pos"], **basis_kw(basis))
    g = gpu_for(param, md, desc, U0)
    before = S.conservation_totals(g)
    t, n, _ = S.ssp33(g)
    after = S.conservation_totals(g)
    assert abs(t - 0.05) < 1e-14 and n > 10
    np.testing.assert_allclose(after, before, rtol=0, atol=1e-13)
    assert after[3] == 0.0  # (rho, rhou, E) and a zero slot
    g.close()


def test_shu_osher_example_run():
    """examples/1D/shu-osher.jl's configuration (Gauss, NodewiseScaledExtrapolation,
    PositivityBound, dt0 1e-4) to T = 0.1: 2001 steps."""
    param, md, bc, desc, U0 = setup(problems.shu_osher, T=0.1)
    o = oracle_for(desc, U0)
    to, no, _ = o.run()
    g = gpu_for(param, md, desc, U0)
    tg, ng, _ = S.ssp33(g)
    assert ng == no and abs(tg - to) <= 1e-12
    assert relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)) <= TOL_RUN
    th = g.get_field(abi.FIELD_THETA_LOCAL, 3)
    assert th.min() < 1.0  # the projection limiter is active at the shock
    g.close()
    o.close()


def test_line_error_against_exact():
    """calculate_error on the device for the Line state against the density wave."""
    param, md, bc, desc, U0 = setup(problems.density_wave_1d, N=3, K=16, T=0.02,
                                    rhs_limiter=LIMITERS["pos"])
    g = gpu_for(param, md, desc, U0)
    S.ssp33(g)
    err = S.calculate_error(None, g, problems.density_wave_1d_exact)
    assert 0 < err.L1err < 1e-5 and err.L2err < 1e-5 and err.Linferr < 1e-4
    g.close()


@pytest.mark.parametrize("N", [1, 3, 5])
@pytest.mark.parametrize("basis", ["lobatto", "gauss"])
@pytest.mark.parametrize("limiter", ["pos", "cell", "relaxed-cell", "minent", "tvd-minent", "pos+hennemann",
                                     "zhang-shu+hennemann"])
def test_line_team_layout_gives_the_same_bits(limiter, basis, N):
    """The team layout of the Line kernels (a team of lanes per element, the default below
    2048 elements; the face projection's bisection speculative across a warp) against one
    thread per element: the state, the right-hand sides, the face fluxes, theta, the subcell
    factors and the stage minima after ten steps, bitwise."""
    if basis == "gauss" and limiter in CELL:
        pytest.skip("no cell-entropy bound on Gauss nodes in 1D")
    param, md, bc, desc, U0 = setup(problems.leblanc, N=N, K=50, T=0.05, rhs_limiter=LIMITERS[limiter],
                                    **basis_kw(basis))
    out = {}
    for layout in (abi.LAYOUT_FLAT, abi.LAYOUT_TEAM):
        g = gpu_for(param, md, desc, U0)
        g.set_layout(layout)
        assert g.layout() == layout
        t = param.timestepping_param.t0
        for _ in range(10):
            t, _ = S.ssp33_step(g, t)
        fields = [g.get_field(abi.FIELD_UQ), g.get_field(abi.FIELD_RHSU), g.get_field(abi.FIELD_RHSH),
                  g.get_field(abi.FIELD_RHSL), g.get_field(abi.FIELD_BF_L), g.get_field(abi.FIELD_BF_H)]
        fields += [g.get_field(abi.FIELD_THETA_LOCAL, s) for s in (1, 2, 3)]
        mins = np.zeros(6)
        g._check(g.lib.p2de_stage_minima(g.handle, abi.dptr(mins)))
        fields.append(mins)
        if isinstance(LIMITERS[limiter], SubcellLimiter):
            fields += [g.get_field(abi.FIELD_L_LOCAL, s) for s in (1, 2, 3)]
        else:
            fields += [g.get_field(abi.FIELD_L, s) for s in (1, 2, 3)]
        out[layout] = (t, fields)
        g.close()
    assert out[abi.LAYOUT_FLAT][0] == out[abi.LAYOUT_TEAM][0]
    for a, b in zip(out[abi.LAYOUT_FLAT][1], out[abi.LAYOUT_TEAM][1]):
        np.testing.assert_array_equal(a, b)


def test_line_layout_default_and_values():
    param, md, bc, desc, U0 = setup(problems.shu_osher, N=1, K=2048)
    g = gpu_for(param, md, desc, U0)
    assert g.layout() == abi.LAYOUT_FLAT  # from 2048 elements one thread per element is faster
    with pytest.raises(abi.P2deError):
        g.set_layout(abi.LAYOUT_LINES_PER_WARP)
    g.close()
    param, md, bc, desc, U0 = setup(problems.shu_osher, N=1, K=64)
    g = gpu_for(param, md, desc, U0)
    assert g.layout() == abi.LAYOUT_TEAM
    g.close()
