"""GPU parity of the limiter variants beyond the positivity / cell-entropy / TVD bounds:
ZhangShuLimiter (zhangshu.jl), the min-entropy bounds with their bisection
(limiter_utils.jl:19-50, subcell.jl:21-72) and the relaxed bounds (subcell.jl:750-753,
937-956), against the FP64 oracle on the same seeded inputs, and the reference's own
smoke-test matrix (test/test_smoke.jl:44-52) run to its final time.
"""
import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.types import (
    HennemannShockCapture,
    NoShockCapture,
    PositivityAndCellEntropyBound,
    PositivityAndMinEntropyBound,
    PositivityAndRelaxedCellEntropyBound,
    PositivityAndRelaxedMinEntropyBound,
    PositivityBound,
    SubcellLimiter,
    TVDAndMinEntropyBound,
    TVDAndRelaxedCellEntropyBound,
    TVDAndRelaxedMinEntropyBound,
    ZhangShuLimiter,
)

from conftest import relerr
from helpers import setup
from test_gpu_parity import TOL, compare_rhs, gpu_for, intended_cell_tol, oracle_for

pytestmark = pytest.mark.gpu

# The cell-entropy repair under the intended bounds reacts to rounding-level entropy
# production; its relaxed form likewise: such cases are compared at TOL or ten times the
# oracle's own one-ulp sensitivity (test_gpu_parity.intended_cell_tol).
# The min-entropy bisection decides phi(uL + l P) >= Lphi - POSTOL on a grid of 21
# halvings: one comparison that rounds the other way (pow is not correctly rounded on
# either side) moves l by up to lpos 2^-21, and where a stencil is nearly flat (P near
# zero, phi at the threshold) it flips a factor between 0 and 1 while rhsU moves by
# rounding only. The oracle against itself, with a one-ulp change of the initial state:
# 75 interior factors of a TVD-min RHS flip while its rhsU moves by 6e-16; the
# smoke-test vortex runs (2-3 steps) differ by 6e-12 (N = 1) to 1e-8 (relaxed, N = 4).
# Single RHS evaluations are compared at TOL without their interior factors; runs at
# ten times the largest of those self-differences.
TOL_MIN_ENTROPY = 1e-7

MIN_BOUNDS = {
    "min": PositivityAndMinEntropyBound(),
    "relaxed-min": PositivityAndRelaxedMinEntropyBound(),
    "tvd-min": TVDAndMinEntropyBound(),
    "tvd-relaxed-min": TVDAndRelaxedMinEntropyBound(),
}
RELAXED_CELL = {
    "relaxed-cell": PositivityAndRelaxedCellEntropyBound(beta=0.5),
    "tvd-relaxed-cell": TVDAndRelaxedCellEntropyBound(beta=0.5),
}


def run_steps(param, md, desc, U0, nsteps):
    o = oracle_for(desc, U0)
    g = gpu_for(param, md, desc, U0)
    to, tg = param.timestepping_param.t0, param.timestepping_param.t0
    for _ in range(nsteps):
        to, _ = o.step(to)
        tg, _ = S.ssp33_step(g, tg)
    return o, g, to, tg


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("shock", [False, True])
def test_zhang_shu_rhs(N, shock):
    sc = HennemannShockCapture(a=0.5, c=1.8) if shock else NoShockCapture()
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=N, Kx=6, Ky=5, T=0.2, seed=4,
                                    rhs_limiter=ZhangShuLimiter(shockcapture=sc))
    # the limiter's dt is the stage-1 CFL dt0 of SSP33! (0.1), where the bounds bind
    for nstage in (1, 2):
        compare_rhs(param, md, desc, U0, dt=0.1, nstage=nstage)
    o = oracle_for(desc, U0)
    g = gpu_for(param, md, desc, U0)
    o.rhs(0.0, 0.1, 3)
    S.rhs_bang(None, g, None, p2de.TimeParam(0.0, 0.1, 3))
    Lg, Lo = g.get_field(abi.FIELD_L, 3), o.get_field(abi.FIELD_L, 3)
    assert Lg.shape == (desc.K,)
    assert np.all((Lg >= 0) & (Lg <= 1)) and Lg.min() < 1  # the limiter is active
    np.testing.assert_allclose(Lg, Lo, rtol=1e-12, atol=1e-15)
    g.close()
    o.close()


@pytest.mark.parametrize("N", [1, 3, 5])
def test_zhang_shu_steps(N):
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=N, Kx=6, Ky=5, T=0.2, seed=7,
                                    rhs_limiter=ZhangShuLimiter())
    o, g, to, tg = run_steps(param, md, desc, U0, 5)
    assert abs(tg - to) <= 1e-13 * abs(to)
    assert relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)) <= TOL
    g.close()
    o.close()


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("bound", list(MIN_BOUNDS))
def test_min_entropy_rhs(N, bound):
    """Stage 1 at t0 (the relaxed bounds take the initial minimum of phi there), then a
    later stage that reads it."""
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=N, Kx=6, Ky=5, T=0.2, seed=4, bound=MIN_BOUNDS[bound])
    compare_rhs(param, md, desc, U0, dt=1e-3, nstage=1, interior_L=False)
    o = oracle_for(desc, U0)
    g = gpu_for(param, md, desc, U0)
    for ns in (1, 2):
        o.rhs(0.0, 1e-3, ns)
        S.rhs_bang(None, g, None, p2de.TimeParam(0.0, 1e-3, ns))
        assert relerr(g.get_field(abi.FIELD_RHSU), o.get_field(abi.FIELD_RHSU)) <= TOL
    L = g.get_field(abi.FIELD_L_LOCAL, 2)
    assert np.all((L >= 0) & (L <= 1)) and L.min() < 1
    g.close()
    o.close()


@pytest.mark.parametrize("bound", list(MIN_BOUNDS))
@pytest.mark.parametrize("N", [2, 4])
def test_min_entropy_steps(N, bound):
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=N, Kx=6, Ky=5, T=0.2, seed=7, bound=MIN_BOUNDS[bound])
    o, g, to, tg = run_steps(param, md, desc, U0, 4)
    assert abs(tg - to) <= 1e-13 * abs(to)
    assert relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)) <= TOL_MIN_ENTROPY
    g.close()
    o.close()


@pytest.mark.parametrize("refsem", [True, False])
@pytest.mark.parametrize("bound", list(RELAXED_CELL))
@pytest.mark.parametrize("N", [2, 3, 5])
def test_relaxed_cell_entropy_rhs(N, bound, refsem):
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=N, Kx=6, Ky=6, T=0.1, bound=RELAXED_CELL[bound],
                                    reference_semantics=refsem)
    tol = TOL if refsem else intended_cell_tol(desc, U0, 0.0, 2e-4, 2)
    compare_rhs(param, md, desc, U0, dt=2e-4, nstage=2, tol=tol)


# the reference's smoke test (test/test_smoke.jl:44-52): isentropic vortex, K = (5, 5),
# N = 1..4, T = 2e-2, CFL 1, dt0 1e-2, each limiter run to the final time
SMOKE_LIMITERS = {
    "zhang-shu": ZhangShuLimiter(),
    "positivity": SubcellLimiter(bound=PositivityBound()),
    "positivity-hennemann": SubcellLimiter(bound=PositivityBound(), shockcapture=HennemannShockCapture()),
    "min-entropy": SubcellLimiter(bound=PositivityAndMinEntropyBound()),
    "relaxed-min-entropy": SubcellLimiter(bound=PositivityAndRelaxedMinEntropyBound()),
    "cell-entropy": SubcellLimiter(bound=PositivityAndCellEntropyBound()),
    "relaxed-cell-entropy": SubcellLimiter(bound=PositivityAndRelaxedCellEntropyBound(beta=0.5)),
}


@pytest.mark.parametrize("refsem", [True, False])
@pytest.mark.parametrize("limiter", list(SMOKE_LIMITERS))
def test_reference_smoke_matrix(limiter, refsem):
    for N in (1, 2, 3, 4):
        param, ic, bcf, exact = problems.isentropic_vortex(N=N, Kx=5, Ky=5, T=2e-2, rhs_limiter=SMOKE_LIMITERS[limiter],
                                                            reference_semantics=refsem)
        md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
        bc = bcf(param, md)
        desc = S.make_descriptor(param, md, bc)
        U0 = S.evaluate_initial_condition(param, md, ic)
        o = oracle_for(desc, U0)
        to, no, _ = o.run()
        g = gpu_for(param, md, desc, U0)
        tg, ng, _ = S.ssp33(g)
        assert ng == no and abs(tg - to) <= 1e-13 * abs(to)
        tol = TOL
        if "cell" in limiter and not refsem:
            # ten times the oracle's own change over the run under a one-ulp change of U0
            o1 = oracle_for(desc, np.nextafter(U0, np.inf))
            o1.run()
            tol = max(TOL, 10.0 * relerr(o1.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)))
            o1.close()
        elif "min-entropy" in limiter:
            tol = TOL_MIN_ENTROPY
        e = relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ))
        assert e <= tol, (N, e)
        g.close()
        o.close()
