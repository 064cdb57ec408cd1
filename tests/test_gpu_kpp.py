"""GPU parity of the KPP equation (src/math/KPP.jl; examples/2D/KPP.jl) and of the
LaxFriedrichsOnProjectedVal low-order flux (low_order_graph_viscosity.jl:63-71, 245-318)
against the FP64 oracle: the scalar law carried in the first state component, its
entropy-conservative flux, wavespeed 1, the subcell limiter reduced to the shock-capture
blending factor (subcell.jl:389-402), Zhang-Shu's factor 1 (zhangshu.jl:58-60), and the
projected-flux CFL term alpha lambdaB + |B| ws / 2.
"""
import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.types import (
    HennemannShockCapture,
    LaxFriedrichsOnProjectedVal,
    NoShockCapture,
    PositivityBound,
    SubcellLimiter,
    ZhangShuLimiter,
)

from conftest import relerr
from helpers import setup
from test_gpu_parity import TOL, compare_rhs, gpu_for, oracle_for

pytestmark = pytest.mark.gpu

# KPP's entropy-conservative flux (KPP.jl:25-38) averages only for |uR - uL| < 1e-12;
# just above, (cos uL - cos uR) / (uR - uL) cancels catastrophically, so one ulp of sin/cos
# (glibc in the oracle, CUDA here) becomes a relative flux error up to ~1e-4. After a few
# steps the flat regions beside the disc carry differences in that range, and the oracle
# against itself with a one-ulp change of the state after two steps differs by 5e-9
# (N = 1), 5.5e-8 (N = 3), 9.5e-8 (N = 5) three steps later. Single RHS evaluations are
# compared at TOL; runs at ten times those self-differences.
TOL_KPP_RUN = 1e-6

KPP_LIMITERS = {
    "hennemann": SubcellLimiter(shockcapture=HennemannShockCapture()),
    "no-shock-capture": SubcellLimiter(bound=PositivityBound(), shockcapture=NoShockCapture()),
    "zhang-shu+hennemann": ZhangShuLimiter(shockcapture=HennemannShockCapture()),
}


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("limiter", list(KPP_LIMITERS))
def test_kpp_rhs(N, limiter):
    param, md, bc, desc, U0 = setup(problems.kpp, N=N, Kx=8, Ky=8, T=0.1, rhs_limiter=KPP_LIMITERS[limiter])
    assert np.shape(U0)[-1] == 1
    for ns in (1, 2):
        compare_rhs(param, md, desc, U0, dt=5e-4, nstage=ns)


@pytest.mark.parametrize("N", [1, 3, 5])
def test_kpp_steps(N):
    param, md, bc, desc, U0 = setup(problems.kpp, N=N, Kx=8, Ky=8, T=0.1)
    o = oracle_for(desc, U0)
    g = gpu_for(param, md, desc, U0)
    to, tg = 0.0, 0.0
    for _ in range(5):
        to, _ = o.step(to)
        tg, _ = S.ssp33_step(g, tg)
    assert abs(tg - to) <= 1e-13 * abs(to)
    assert relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)) <= TOL_KPP_RUN
    L = g.get_field(abi.FIELD_L_LOCAL, 3)
    assert L.min() <= 0.5 + 1e-15  # elements on the discontinuity take alphamax
    g.close()
    o.close()


def test_kpp_reference_example_to_final_time():
    """examples/2D/KPP.jl's configuration on a 16 x 16 mesh to T = 0.05 (100 steps)."""
    param, md, bc, desc, U0 = setup(problems.kpp, N=3, Kx=16, Ky=16, T=0.05)
    o = oracle_for(desc, U0)
    to, no, _ = o.run()
    g = gpu_for(param, md, desc, U0)
    tg, ng, _ = S.ssp33(g)
    assert ng == no == 100 and abs(tg - to) <= 1e-13
    assert relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)) <= TOL_KPP_RUN
    g.close()
    o.close()


@pytest.mark.parametrize("N", [2, 3])
@pytest.mark.parametrize("problem", ["riemann", "dmr"])
def test_projected_low_order_flux_euler(N, problem):
    """LaxFriedrichsOnProjectedVal as the low-order flux on LGL nodes (the projection is
    the identity there): same RHS, CFL with alpha lambdaB + |B| ws / 2 per face."""
    from dataclasses import replace

    prob, kw = {"riemann": (problems.riemann2d, dict(Kx=6, Ky=5, T=0.2, seed=4)),
                "dmr": (problems.double_mach_reflection, dict(Kx=16, Ky=4, T=0.2))}[problem]
    param, md, bc, desc, U0 = setup(prob, N=N, **kw)
    param = replace(param, rhs=p2de.ESLimitedLowOrderPos(low_order_surface_flux=LaxFriedrichsOnProjectedVal()))
    desc = S.make_descriptor(param, md, bc)
    compare_rhs(param, md, desc, U0, dt=0.2, nstage=1)
    o = oracle_for(desc, U0)
    g = gpu_for(param, md, desc, U0)
    to, tg = 0.0, 0.0
    for _ in range(3):
        to, _ = o.step(to)
        tg, _ = S.ssp33_step(g, tg)
    assert abs(tg - to) <= 1e-13 * abs(to)
    assert relerr(g.get_field(abi.FIELD_UQ), o.get_field(abi.FIELD_UQ)) <= TOL
    g.close()
    o.close()


def test_kpp_rejects_what_is_not_built():
    from dataclasses import replace

    from p2de.types import GaussCollocation, TVDBound

    param, md, bc, desc, U0 = setup(problems.kpp, N=2, Kx=4, Ky=4, T=0.1)
    with pytest.raises(S.UnsupportedMethod):
        S.lower_param(replace(param, rhs_limiter=SubcellLimiter(bound=TVDBound())), desc.K)
    with pytest.raises(S.UnsupportedMethod):
        S.lower_param(replace(param, approximation_basis=GaussCollocation()), desc.K)
