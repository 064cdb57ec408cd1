"""The cell entropy inequality of the subcell limiter, checked on every stage's output.

enforce_ES_subcell_volume! (subcell.jl:630-744) exists to make, per element and direction,
sum L dvdf <= rhs_es + max(0, sum_dvfbarL - sum_Bpsi) (rhs_es :746-753); the reference's
checker of it is check_subcell_entropy_stability (experimental/entropy-stable-limiting.jl:
790-955, its call commented out at limiter.jl:55). p2de.entropy evaluates both sides with
numpy from the stage's input Uq, f_bar_H, f_bar_L and L_local, independently of the code
that produced them; here they come from the oracle (CPU tests) and from the GPU through the
C ABI (P2DE_FIELD_F_BAR_H/L, L_local; GPU tests), at every stage of three SSP-RK3 steps,
for every cell-entropy bound, both limiter semantics, LGL and Gauss nodes. A planted
violation (factors cut on the faces that lower the entropy production and kept on the
others) shows that the evaluation detects one."""
import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.entropy import cell_entropy_sides, cell_entropy_violation, v_ufun
from p2de.mesh import gauss_rule, gll_rule
from p2de.types import (
    GaussCollocation,
    NodewiseScaledExtrapolation,
    PositivityAndCellEntropyBound,
    PositivityAndRelaxedCellEntropyBound,
    TVDAndCellEntropyBound,
    TVDAndRelaxedCellEntropyBound,
)

from helpers import setup

BOUNDS = {
    "cell": PositivityAndCellEntropyBound(),
    "tvd-cell": TVDAndCellEntropyBound(),
    "relaxed-cell": PositivityAndRelaxedCellEntropyBound(beta=0.5),
    "tvd-relaxed-cell": TVDAndRelaxedCellEntropyBound(beta=0.5),
}

PROBLEMS = {
    "riemann": (problems.riemann2d, dict(N=3, Kx=10, Ky=10, T=0.2, seed=3)),
    "blast": (problems.sedov_lgl, dict(N=3, Kx=16, Ky=16, T=0.05)),
    "dmr": (problems.double_mach_reflection, dict(N=3, Kx=24, Ky=6, T=0.2)),
    "kh": (problems.kelvin_helmholtz, dict(N=3, Kx=8, Ky=8, T=0.1)),
}

GAUSS = dict(approximation_basis=GaussCollocation(), entropyproj_limiter=NodewiseScaledExtrapolation())


def _case(problem, bound, refsem, gauss=False):
    fn, kw = PROBLEMS[problem]
    kw = dict(kw, bound=BOUNDS[bound], reference_semantics=refsem, **(GAUSS if gauss else {}))
    return setup(fn, **kw)


def _weights(param):
    rule = gauss_rule if isinstance(param.approximation_basis, GaussCollocation) else gll_rule
    return rule(param.N)[1]


def _check_kw(param):
    beta = getattr(param.rhs_limiter.bound, "beta", None)
    return {"relaxed_beta": beta} if beta is not None else {}


class _Probe:
    """What SSP33_host_loop reads of a solver."""

    def __init__(self, param, desc):
        self.param, self.desc = param, desc
        self.K, self.Nq, self.N1D = desc.K, desc.Nq, desc.N + 1


def run_and_check(param, md, desc, U0, evaluate, steps=3):
    """Three SSP-RK3 steps (SSP33_host_loop) whose right-hand side is evaluate(U, t, dt,
    nstage) -> (dt, rhsU, f_bar_H, f_bar_L, L_local); after every stage the inequality is
    evaluated on that stage's fields. Returns the worst scaled excess and the stage count."""
    w = _weights(param)
    worst, stages = -np.inf, 0

    def rhs(state, solver, state_param, tp):
        nonlocal worst, stages
        pre = state.preallocation
        dt, rhsU, fH, fL, L = evaluate(pre.Uq, tp.t, tp.dt, tp.nstage)
        pre.rhsU[...] = rhsU.reshape(pre.rhsU.shape)
        wv, _ = cell_entropy_violation(pre.Uq, fH, fL, L, md.geom, param.N, w, param.equation.gamma,
                                       zerotol=param.global_constants.ZEROTOL, **_check_kw(param))
        worst = max(worst, wv)
        stages += 1
        return dt

    probe = _Probe(param, desc)
    S.SSP33_host_loop(S.HostState(probe, U0), probe, None, nsteps=steps, rhs=rhs)
    return worst, stages


def _oracle_evaluate(desc):
    from oracle.binding import Oracle

    o = Oracle(desc)

    def evaluate(U, t, dt, nstage):
        o.set_Uq(U)
        dt = o.rhs(t, dt, nstage)
        return (dt, o.get_field(abi.FIELD_RHSU), o.get_field(abi.FIELD_F_BAR_H), o.get_field(abi.FIELD_F_BAR_L),
                o.get_field(abi.FIELD_L_LOCAL, nstage))

    return evaluate


# ---- CPU: the oracle, and the evaluation itself -----------------------------------------
@pytest.mark.parametrize("problem", ["riemann", "blast"])
@pytest.mark.parametrize("bound", ["cell", "relaxed-cell"])
@pytest.mark.parametrize("refsem", [True, False])
def test_oracle_satisfies_the_cell_entropy_inequality(problem, bound, refsem):
    param, md, bc, desc, U0 = _case(problem, bound, refsem)
    worst, stages = run_and_check(param, md, desc, U0, _oracle_evaluate(desc))
    assert stages == 9 and worst <= 0.0, worst


def test_oracle_satisfies_the_cell_entropy_inequality_on_gauss_nodes():
    param, md, bc, desc, U0 = _case("riemann", "cell", False, gauss=True)
    worst, stages = run_and_check(param, md, desc, U0, _oracle_evaluate(desc))
    assert stages == 9 and worst <= 0.0, worst


def test_a_planted_violation_is_detected():
    """Cut every interior factor whose face lowers the entropy production (dvdf < 0) and keep
    the others at 1: the limited fluxes then produce more entropy than the bound allows.
    (Kelvin-Helmholtz data: their noise makes every element's entropy variables vary.)"""
    param, md, bc, desc, U0 = _case("kh", "cell", False)
    ev = _oracle_evaluate(desc)
    dt, _, fH, fL, L = ev(U0, 0.0, 1e-3, 1)
    w = _weights(param)
    worst, _ = cell_entropy_violation(U0, fH, fL, L, md.geom, param.N, w)
    assert worst <= 0.0
    n, K = param.N + 1, desc.K
    v = v_ufun(np.asarray(U0).reshape(K, n * n, 4), param.equation.gamma)
    fH4 = fH.reshape(2, K, n * (n + 1), 4)
    fL4 = fL.reshape(2, K, n * (n + 1), 4)
    bad = L.reshape(K, 2, n * (n + 1)).copy()
    for d in range(2):
        for a in range(n):
            for b in range(1, n):
                fi, qm, qp = ((b + (n + 1) * a, (b - 1) + n * a, b + n * a) if d == 0
                              else (a + n * b, a + n * (b - 1), a + n * b))
                dvdf = np.sum((v[:, qm] - v[:, qp]) * (fH4[d, :, fi] - fL4[d, :, fi]), axis=-1)
                bad[:, d, fi] = np.where(dvdf < 0, 0.0, 1.0)
    worst, mask = cell_entropy_violation(U0, fH, fL, bad, md.geom, param.N, w)
    assert worst > 1e-6 and mask.sum() >= K // 4, (worst, mask.sum())
    # with every interior factor 1 the volume fluxes are the entropy-conservative ones
    # (sum dvdf = rhs_es up to rounding), with every factor 0 the low-order ones
    for fill in (1.0, 0.0):
        lhs, target, scale = cell_entropy_sides(U0, fH, fL, np.full_like(bad, fill), md.geom, param.N, w)
        assert np.all(lhs - target <= 1e-12 * scale)


# ---- GPU: the same inequality on the GPU's own stage outputs ----------------------------
def _gpu_evaluate(param, md, desc):
    g = S.Solver(param, md, desc)
    st = S.HostState(g, np.zeros((desc.K, desc.Nq, 4)))

    def evaluate(U, t, dt, nstage):
        st.preallocation.Uq[...] = U
        dt = S.rhs_bang(st, g, None, p2de.TimeParam(t, dt, nstage))
        return (dt, st.preallocation.rhsU.copy(), g.get_field(abi.FIELD_F_BAR_H), g.get_field(abi.FIELD_F_BAR_L),
                g.get_field(abi.FIELD_L_LOCAL, nstage))

    return evaluate, g


@pytest.mark.gpu
@pytest.mark.parametrize("problem", list(PROBLEMS))
@pytest.mark.parametrize("bound", list(BOUNDS))
@pytest.mark.parametrize("refsem", [True, False])
def test_gpu_satisfies_the_cell_entropy_inequality(problem, bound, refsem):
    param, md, bc, desc, U0 = _case(problem, bound, refsem)
    ev, g = _gpu_evaluate(param, md, desc)
    worst, stages = run_and_check(param, md, desc, U0, ev)
    g.close()
    assert stages == 9 and worst <= 0.0, worst


@pytest.mark.gpu
@pytest.mark.parametrize("problem", ["riemann", "dmr"])
@pytest.mark.parametrize("bound", ["cell", "tvd-cell"])
@pytest.mark.parametrize("refsem", [True, False])
def test_gpu_satisfies_the_cell_entropy_inequality_on_gauss_nodes(problem, bound, refsem):
    param, md, bc, desc, U0 = _case(problem, bound, refsem, gauss=True)
    ev, g = _gpu_evaluate(param, md, desc)
    worst, stages = run_and_check(param, md, desc, U0, ev)
    g.close()
    assert stages == 9 and worst <= 0.0, worst
