"""The FP64 oracle against mathematical invariants of the reference's scheme and
against the committed golden vectors (CPU only). PARITY UNPINNED: the reference has
no golden vectors of its own for this path (test/test_smoke.jl asserts nothing)."""
from pathlib import Path

import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.types import (
    HennemannShockCapture,
    PositivityAndCellEntropyBound,
    PositivityAndMinEntropyBound,
    PositivityAndRelaxedCellEntropyBound,
    PositivityAndRelaxedMinEntropyBound,
    PositivityBound,
    SubcellLimiter,
    TVDAndCellEntropyBound,
    TVDAndMinEntropyBound,
    TVDAndRelaxedMinEntropyBound,
    TVDBound,
    ZhangShuLimiter,
    GaussCollocation,
    NodewiseScaledExtrapolation,
)

from conftest import relerr
from helpers import setup
from oracle.binding import Oracle, fluxes, fS, logmean

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_gll_rule(N):
    r, w = p2de.gll_rule(N)
    assert abs(w.sum() - 2.0) < 1e-14
    np.testing.assert_allclose(r, -r[::-1], atol=1e-15)
    for k in range(2 * N):  # exact for degree <= 2N - 1
        exact = (1 - (-1) ** (k + 1)) / (k + 1)
        assert abs(np.sum(w * r**k) - exact) < 1e-13


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_operator_invariants_and_nnz(N):
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=N, Kx=2, Ky=2, T=0.1)
    o = Oracle(desc, nthreads=1)
    n = N + 1
    Nq, Nfp = n * n, 4 * n
    Nh = Nq + Nfp
    nh, nl = o.nnz_counts()
    assert nh == n * n * (n - 1) + Nfp  # within-line pairs + face pairs (64 for N=3)
    assert nl == 2 * n * (n - 1)
    for which in (3, 4):
        S_ = o.operator(which).reshape(Nh, Nh, order="F")
        np.testing.assert_allclose(S_, -S_.T, atol=1e-14)
        rows = S_.sum(axis=1)
        # SBP: volume rows of the hybridized operator sum to zero, face rows to -B
        assert np.max(np.abs(rows[:Nq])) < 1e-13
        B = -rows[Nq:]
        w = p2de.gll_rule(N)[1]
        side = np.arange(Nfp) // n
        expect = np.zeros(Nfp)
        if which == 3:
            expect[side == 0], expect[side == 1] = -np.tile(w, 1), w
        else:
            expect[side == 2], expect[side == 3] = -np.tile(w, 1), w
        np.testing.assert_allclose(B, expect, atol=1e-14)


def test_fS_consistency_and_symmetry():
    g = 1.4
    rng = np.random.default_rng(0)
    for _ in range(50):
        rho, u, v, p = rng.uniform(0.2, 3), rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(0.1, 5)
        beta = rho / (2 * p)
        U6 = np.array([rho, u, v, beta, np.log(rho), np.log(beta)])
        E = p / (g - 1) + 0.5 * rho * (u * u + v * v)
        f = fluxes(g, [rho, rho * u, rho * v, E])
        np.testing.assert_allclose(fS(g, U6, U6), f, rtol=1e-13, atol=1e-13)
        rho2, u2, v2, p2 = rng.uniform(0.2, 3), rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(0.1, 5)
        b2 = rho2 / (2 * p2)
        V6 = np.array([rho2, u2, v2, b2, np.log(rho2), np.log(b2)])
        np.testing.assert_allclose(fS(g, U6, V6), fS(g, V6, U6), rtol=1e-14, atol=1e-14)


def test_logmean_reference_series():
    """The reference's small-|f| series (compressible_Navier_Stokes.jl:315-317) is kept
    verbatim; it departs from the exact log mean by up to ~1.1e-9 near |f| = 1e-4."""
    for f in [1e-6, 5e-5, 9.9e-5]:
        aL = 1.0
        aR = aL * (1 + f / 2) / (1 - f / 2)  # (aR-aL)/avg = f
        exact = (aR - aL) / (np.log(aR) - np.log(aL))
        got = logmean(aL, aR)
        assert abs(got - exact) / exact < 1.2e-9
    got = logmean(1.0, 2.0)
    assert abs(got - 1.0 / np.log(2.0)) < 1e-15


def _constant_state_problem(N=3):
    param, ic, bcf = problems.kelvin_helmholtz(N=N, Kx=4, Ky=3, T=0.1)

    def constant(param, x, y):
        return problems.primitive_to_conservative(param.equation, (1.3 + 0 * x, 0.4 + 0 * x, -0.7 + 0 * x, 2.1 + 0 * x))

    return param, constant, bcf


@pytest.mark.parametrize("N", [1, 3, 5])
def test_free_stream_preservation(N):
    param, ic, bcf = _constant_state_problem(N)
    md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
    desc = S.make_descriptor(param, md, bcf(param, md))
    o = Oracle(desc, nthreads=1)
    o.set_Uq(S.evaluate_initial_condition(param, md, ic))
    o.rhs(0.0, 1e-3, 1)
    for f in (abi.FIELD_RHSU, abi.FIELD_RHSL, abi.FIELD_RHSH):
        assert np.max(np.abs(o.get_field(f))) < 1e-11


def test_free_stream_on_rotated_elements():
    """Affine elements with sxJ, ryJ != 0 (every node rotated): a constant state stays
    constant (the general geometric path of the oracle)."""
    param, ic, bcf = _constant_state_problem(N=3)
    md = p2de.mesh.rotated(p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR), 0.4)
    desc = S.make_descriptor(param, md, bcf(param, md))
    U0 = S.evaluate_initial_condition(param, md, ic)
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    o.rhs(0.0, 1e-3, 1)
    assert np.abs(o.get_field(abi.FIELD_RHSU)).max() < 1e-12


def test_conservation_periodic():
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=6, Ky=6, T=0.1)
    o = Oracle(desc, nthreads=2)
    o.set_Uq(U0)
    w = p2de.gll_rule(3)[1]
    wq = np.outer(w, w).ravel()  # wq[ir + 4 is] = w[ir] w[is]

    def total():
        U = o.get_field(abi.FIELD_UQ).reshape(desc.K, 16, 4)
        return np.einsum("k,i,kic->c", md.geom[:, 0], wq, U)

    c0 = total()
    t = 0.0
    for _ in range(10):
        t, _ = o.step(t)
    c1 = total()
    np.testing.assert_allclose(c1, c0, rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("refsem", [True, False])
@pytest.mark.parametrize("bound", [PositivityBound(), PositivityAndCellEntropyBound(), TVDBound(), TVDAndCellEntropyBound()])
def test_positivity_and_factor_range(refsem, bound):
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=8, Ky=8, T=0.2, seed=2, bound=bound, reference_semantics=refsem)
    o = Oracle(desc, nthreads=2)
    o.set_Uq(U0)
    t = 0.0
    g = 1.4
    for _ in range(8):
        t, _ = o.step(t)
        U = o.get_field(abi.FIELD_UQ).reshape(-1, 4)
        rhoe = U[:, 3] - 0.5 * (U[:, 1] ** 2 + U[:, 2] ** 2) / U[:, 0]
        assert U[:, 0].min() > 0 and rhoe.min() > 0
        for s in (1, 2, 3):
            L = o.get_field(abi.FIELD_L_LOCAL, s)
            assert np.all((L >= 0) & (L <= 1))


def tvd_bounds_np(md, N, rhoL):
    """low_order_stencil (limiter_utils.jl:222-231) min/max of rhoL, restated with numpy
    on the mesh's mapP (q2fq: the r-face first at corners)."""
    n = N + 1
    K = rhoL.shape[0]
    Nfp = 4 * n
    mapP = md.mapP.reshape(K, Nfp) - 1
    fq2q = np.concatenate([n * np.arange(n), N + n * np.arange(n), np.arange(n), np.arange(n) + n * N])
    lb, ub = rhoL.copy(), rhoL.copy()
    for k in range(K):
        for q in range(n * n):
            i, j = q % n, q // n
            faces = ([j] if i == 0 else []) + ([n + j] if i == N else []) + ([2 * n + i] if j == 0 else []) + ([3 * n + i] if j == N else [])

            def across(direction):
                f = faces[0] if len(faces) == 1 else faces[direction - 1]
                lin = mapP[k, f]
                return lin // Nfp, fq2q[lin % Nfp]

            st = [(k, q - 1) if i > 0 else across(1), (k, q + 1) if i < N else across(1),
                  (k, q - n) if j > 0 else across(2), (k, q + n) if j < N else across(2)]
            for kk, qq in st:
                lb[k, q] = min(lb[k, q], rhoL[kk, qq])
                ub[k, q] = max(ub[k, q], rhoL[kk, qq])
    return lb, ub


def test_tvd_bounds_hold_after_a_stage():
    """TVDBound with the intended bounds: the stage-1 update's density stays within the
    min/max of the low-order density over each node's stencil (subcell.jl:112-141)."""
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=6, Ky=5, T=0.2, seed=5, bound=TVDBound(),
                                    reference_semantics=False)
    o = Oracle(desc, nthreads=2)
    o.set_Uq(U0)
    dt = 2e-3
    o.rhs(0.0, dt, 2)
    rhoL = (U0[..., 0] + dt * o.get_field(abi.FIELD_RHSL).reshape(desc.K, -1, 4)[..., 0])
    lb, ub = tvd_bounds_np(md, param.N, rhoL)
    rho1 = U0[..., 0] + dt * o.get_field(abi.FIELD_RHSU).reshape(desc.K, -1, 4)[..., 0]
    tol = 1e-12 * np.abs(rho1).max()
    assert np.all(rho1 >= lb - tol) and np.all(rho1 <= ub + tol)
    L = o.get_field(abi.FIELD_L_LOCAL, 2)
    assert L.min() < 1.0  # the bounds are active somewhere


def with_shock_capture(param, a=0.5, c=1.8):
    from dataclasses import replace

    return replace(param, rhs_limiter=SubcellLimiter(bound=param.rhs_limiter.bound,
                                                      shockcapture=HennemannShockCapture(a=a, c=c)))


def test_shock_capture_blending_of_a_free_stream():
    """A constant state has only the constant mode: smoothness 0, so alpha = alphaE0 and
    every factor is 1 - 1e-4 (shock_capture.jl:118-137) when no bound is active."""
    from dataclasses import replace

    param, ic, bcf = _constant_state_problem(N=3)
    param = replace(with_shock_capture(param), reference_semantics=False)
    md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
    bc = bcf(param, md)
    desc = S.make_descriptor(param, md, bc)
    U0 = S.evaluate_initial_condition(param, md, ic)
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    o.rhs(0.0, 1e-3, 2)
    L = o.get_field(abi.FIELD_L_LOCAL, 2)
    np.testing.assert_allclose(L, 1.0 - 1.0 / (1.0 + 9999.0), rtol=1e-14)


def test_shock_capture_caps_factors_at_shocks():
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=8, Ky=8, T=0.2, seed=2, reference_semantics=False)
    o0 = Oracle(desc, nthreads=2)
    o0.set_Uq(U0)
    o0.rhs(0.0, 1e-3, 2)
    L0 = o0.get_field(abi.FIELD_L_LOCAL, 2).reshape(desc.K, -1)
    ps = with_shock_capture(param)
    o = Oracle(S.make_descriptor(ps, md, bc), nthreads=2)
    o.set_Uq(U0)
    o.rhs(0.0, 1e-3, 2)
    L = o.get_field(abi.FIELD_L_LOCAL, 2).reshape(desc.K, -1)
    assert np.all(L <= L0 + 1e-15) and np.all(L >= 0)
    Lmax = L.max(axis=1)
    assert Lmax.min() <= 0.5 + 1e-15  # elements at the discontinuities get alphamax
    assert Lmax.max() > 0.99          # smooth elements are barely capped


def _phi(U, gamma=1.4):
    U = np.reshape(U, (-1, 4))
    rhoe = U[:, 3] - 0.5 * (U[:, 1] ** 2 + U[:, 2] ** 2) / U[:, 0]
    return rhoe * U[:, 0] ** (-gamma)


MIN_ENTROPY_BOUNDS = [PositivityAndMinEntropyBound(), PositivityAndRelaxedMinEntropyBound(), TVDAndMinEntropyBound(),
                      TVDAndRelaxedMinEntropyBound()]


@pytest.mark.parametrize("bound", MIN_ENTROPY_BOUNDS, ids=lambda b: type(b).__name__)
def test_min_entropy_bound_keeps_the_minimum_of_phi(bound):
    """One forward-Euler stage with the limited RHS: every node is the average of four
    states with phi >= Lphi - POSTOL (limiter_utils.jl:43-50), and {phi >= c} is convex, so
    min phi does not fall below the initial min (the lower bound of every stencil, for the
    relaxed bounds too, whose Lphi blends the local min with the global one). The
    positivity bound alone lets it fall on the same data."""
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=8, Ky=8, T=0.2, seed=4, bound=bound,
                                    reference_semantics=False)
    phi0 = _phi(U0).min()
    o = Oracle(desc, nthreads=2)
    o.set_Uq(U0)
    dt = 2e-3
    o.rhs(0.0, dt, 1)
    U1 = np.ravel(U0) + dt * o.get_field(abi.FIELD_RHSU)
    assert _phi(U1).min() >= phi0 * (1 - 1e-12)
    L = o.get_field(abi.FIELD_L_LOCAL, 1)
    assert np.all((L >= 0) & (L <= 1)) and L.min() < 1
    o.close()
    pp, _, _, pdesc, _ = setup(problems.riemann2d, N=3, Kx=8, Ky=8, T=0.2, seed=4, bound=PositivityBound(),
                               reference_semantics=False)
    o = Oracle(pdesc, nthreads=2)
    o.set_Uq(U0)
    o.rhs(0.0, dt, 1)
    assert (np.ravel(U0) + dt * o.get_field(abi.FIELD_RHSU)).size and _phi(np.ravel(U0) + dt * o.get_field(abi.FIELD_RHSU)).min() < phi0 * (1 - 1e-3)
    o.close()


@pytest.mark.parametrize("limiter", [ZhangShuLimiter(), SubcellLimiter(bound=PositivityAndMinEntropyBound()),
                                     SubcellLimiter(bound=TVDAndRelaxedMinEntropyBound())],
                         ids=["zhang-shu", "min-entropy", "tvd-relaxed-min-entropy"])
def test_five_name_bounds_ignore_reference_semantics(limiter):
    """ZhangShuLimiter's 4-tuple and the min-entropy bounds' 5-tuple are read with as many
    names as they have (limiter_utils.jl:4-8,19-24): the destructuring quirk does not
    apply, so both settings give the same bits."""
    out = []
    for refsem in (True, False):
        param, md, bc, desc, U0 = setup(problems.riemann2d, N=2, Kx=6, Ky=6, T=0.2, seed=5, rhs_limiter=limiter,
                                        reference_semantics=refsem)
        o = Oracle(desc, nthreads=2)
        o.set_Uq(U0)
        t = 0.0
        for _ in range(2):
            t, _ = o.step(t)
        out.append(o.get_field(abi.FIELD_UQ))
        o.close()
    assert np.array_equal(out[0], out[1])


def test_zhang_shu_blends_low_and_high_order():
    """rhsU = (1 - l) rhsL + l rhsH per element with l = L[k] (zhangshu.jl:22-23), l in
    [0, 1], below 1 at the discontinuities and 1 in the flat quadrants. The limiter's dt
    is the one SSP33! passes at stage 1, CFL dt0 (0.1 here), before the positivity CFL."""
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=6, Ky=5, T=0.2, seed=4, rhs_limiter=ZhangShuLimiter())
    o = Oracle(desc, nthreads=2)
    o.set_Uq(U0)
    o.rhs(0.0, 0.1, 2)
    L = o.get_field(abi.FIELD_L, 2)
    assert L.shape == (desc.K,) and np.all((L >= 0) & (L <= 1))
    assert L.min() < 0.5 and L.max() == 1.0
    rL = o.get_field(abi.FIELD_RHSL).reshape(desc.K, -1)
    rH = o.get_field(abi.FIELD_RHSH).reshape(desc.K, -1)
    rU = o.get_field(abi.FIELD_RHSU).reshape(desc.K, -1)
    np.testing.assert_allclose(rU, (1 - L)[:, None] * rL + L[:, None] * rH, rtol=1e-13, atol=1e-13 * np.abs(rH).max())
    o.close()


def test_relaxed_cell_entropy_limits():
    """beta = 0 leaves the cell-entropy target unchanged (rhs_es, subcell.jl:746-753)."""
    from dataclasses import replace

    res = []
    for bound in (PositivityAndCellEntropyBound(), PositivityAndRelaxedCellEntropyBound(beta=0.0)):
        param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=6, Ky=6, T=0.1, bound=bound,
                                        reference_semantics=False)
        o = Oracle(desc, nthreads=2)
        o.set_Uq(U0)
        o.rhs(0.0, 2e-4, 2)
        res.append(o.get_field(abi.FIELD_RHSU))
        o.close()
    assert np.array_equal(res[0], res[1])


SMOKE_LIMITERS = [ZhangShuLimiter(), SubcellLimiter(bound=PositivityBound()),
                  SubcellLimiter(bound=PositivityBound(), shockcapture=HennemannShockCapture()),
                  SubcellLimiter(bound=PositivityAndMinEntropyBound()),
                  SubcellLimiter(bound=PositivityAndRelaxedMinEntropyBound()),
                  SubcellLimiter(bound=PositivityAndCellEntropyBound()),
                  SubcellLimiter(bound=PositivityAndRelaxedCellEntropyBound(beta=0.5))]


@pytest.mark.parametrize("limiter", SMOKE_LIMITERS, ids=lambda l: type(l).__name__ + (
    "" if isinstance(l, ZhangShuLimiter) else "-" + type(l.bound).__name__ + "-" + type(l.shockcapture).__name__))
def test_reference_smoke_matrix_runs(limiter):
    """test/test_smoke.jl:44-79: every limiter of the reference's smoke test, N = 1..4 on
    the 5 x 5 vortex, runs to T = 2e-2 with a positive state and the vortex near its
    exact position (the reference's test asserts nothing)."""
    for N in (1, 2, 3, 4):
        param, ic, bcf, exact = problems.isentropic_vortex(N=N, Kx=5, Ky=5, T=2e-2, rhs_limiter=limiter)
        md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
        desc = S.make_descriptor(param, md, bcf(param, md))
        o = Oracle(desc, nthreads=2)
        o.set_Uq(S.evaluate_initial_condition(param, md, ic))
        t, n, _ = o.run()
        assert abs(t - 2e-2) < 1e-14 and n > 0
        U = o.get_field(abi.FIELD_UQ).reshape(-1, 4)
        assert U[:, 0].min() > 0 and _phi(U).min() > 0
        Ue = S.evaluate_initial_condition(
            param, md, lambda prm, x, y: problems.primitive_to_conservative(prm.equation, exact(prm.equation, x, y, t)))
        assert np.abs(U - np.reshape(Ue, U.shape))[:, 0].max() < 0.2
        o.close()


GAUSS = dict(approximation_basis=GaussCollocation(), entropyproj_limiter=NodewiseScaledExtrapolation())


@pytest.mark.parametrize("N", [1, 2, 3, 4])
def test_gauss_free_stream_preservation(N):
    """GaussCollocation (init.jl:83-131): a constant state stays constant; the face
    extrapolation reproduces constants, theta stays 1."""
    param, md, bc, desc, U0 = setup(problems.isentropic_vortex, N=N, Kx=4, Ky=4, T=0.01, strength=0.0,
                                    rhs_limiter=SubcellLimiter(bound=PositivityBound()), **GAUSS)
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    o.rhs(0.0, 1e-3, 1)
    assert np.abs(o.get_field(abi.FIELD_RHSU)).max() < 1e-12
    assert np.all(o.get_field(abi.FIELD_THETA_LOCAL, 1) == 1.0)
    o.close()


def test_gauss_conservation_with_limited_projection():
    """theta Vf + (1 - theta) Vf_low keeps the partition of unity of each face row, so the
    limited lift conserves mass, momentum and energy on a periodic mesh."""
    param, md, bc, desc, U0 = setup(problems.isentropic_vortex, N=3, Kx=5, Ky=5, T=0.05,
                                    rhs_limiter=SubcellLimiter(bound=PositivityBound()), **GAUSS)
    from p2de.mesh import gauss_rule

    _, w = gauss_rule(3)
    wq = np.outer(w, w).ravel()
    J = md.geom[:, 0]
    tot = lambda U: np.einsum("k,i,kic->c", J, wq, np.reshape(U, (desc.K, -1, 4)))
    o = Oracle(desc, nthreads=2)
    o.set_Uq(U0)
    t = 0.0
    for _ in range(4):
        t, _ = o.step(t)
    assert o.get_field(abi.FIELD_THETA_LOCAL, 1).min() < 1.0  # the limiter is active
    np.testing.assert_allclose(tot(o.get_field(abi.FIELD_UQ)), tot(U0), rtol=1e-13, atol=1e-12)
    o.close()


def test_gauss_converges_faster_than_lobatto():
    """Zhang-Shu on the smooth vortex (examples/convergence/isentropic-vortex-convergence.jl
    runs this pairing): the Gauss error is below the LGL one and falls at a high rate."""
    errs = {}
    for basis in ("lobatto", "gauss"):
        errs[basis] = []
        for Kx in (4, 8):
            kw = dict(GAUSS) if basis == "gauss" else {}
            param, ic, bcf, ex = problems.isentropic_vortex(N=3, Kx=Kx, Ky=Kx, T=0.3, strength=1.0, CFL=0.25, dt0=0.3,
                                                            rhs_limiter=ZhangShuLimiter(), **kw)
            md = S.mesh_for(param)
            desc = S.make_descriptor(param, md, bcf(param, md))
            o = Oracle(desc, nthreads=2)
            o.set_Uq(S.evaluate_initial_condition(param, md, ic))
            t, _, _ = o.run()
            U = o.get_field(abi.FIELD_UQ).reshape(-1, 4)
            Ue = S.evaluate_initial_condition(
                param, md, lambda prm, x, y: problems.primitive_to_conservative(prm.equation, ex(prm.equation, x, y, t)))
            errs[basis].append(np.abs(U - np.reshape(Ue, U.shape))[:, 0].max())
            o.close()
    assert errs["gauss"][1] < errs["lobatto"][1]
    assert np.log2(errs["gauss"][0] / errs["gauss"][1]) > 2.0


def test_gauss_mesh_face_points():
    """Face nodes sit at the face Gauss points, not at volume nodes; periodic partners
    coincide up to the period."""
    from p2de.mesh import gauss_rule

    md = p2de.make_periodic(p2de.uniform_mesh(3, 3, 2, (0.0, 0.0), (3.0, 2.0), basis="gauss"))
    r, w = gauss_rule(3)
    assert abs(w.sum() - 2.0) < 1e-14 and np.all(np.abs(r) < 1)
    xf, yf = md.xf.ravel(), md.yf.ravel()
    mP = md.mapP.ravel() - 1
    assert np.all((np.abs(xf - xf[mP]) < 1e-12) | (np.abs(np.abs(xf - xf[mP]) - 3.0) < 1e-12))
    assert np.all((np.abs(yf - yf[mP]) < 1e-12) | (np.abs(np.abs(yf - yf[mP]) - 2.0) < 1e-12))
    assert np.allclose(md.xf[0, :4], 0.0)  # face r = -1 of the first element
    d = np.hypot(md.xf[0][:, None] - md.x[0][None, :], md.yf[0][:, None] - md.y[0][None, :])
    assert d.min() > 1e-3  # no face point is a node


def test_kpp_conserves_and_keeps_constants():
    """KPP (src/math/KPP.jl, examples/2D/KPP.jl): a constant state has no RHS; the
    reference example's discontinuous data conserve the integral of u over periodic
    steps, and the subcell factors are the blending factors (alphamax 1/2 on the disc's
    edge, subcell.jl:389-402)."""
    param, md, bc, desc, U0 = setup(problems.kpp, N=3, Kx=8, Ky=8, T=0.05)
    o = Oracle(desc, nthreads=2)
    o.set_Uq(np.full_like(U0, 1.3))
    o.rhs(0.0, 5e-4, 1)
    assert np.abs(o.get_field(abi.FIELD_RHSU)).max() < 1e-13
    o.set_Uq(U0)
    from p2de.mesh import gll_rule

    w = np.outer(*(2 * [gll_rule(3)[1]])).ravel()
    tot = lambda U: np.einsum("k,i,ki->", md.geom[:, 0], w, np.reshape(U, (desc.K, -1)))
    t = 0.0
    for _ in range(5):
        t, _ = o.step(t)
    assert abs(tot(o.get_field(abi.FIELD_UQ)) - tot(U0)) <= 1e-13 * abs(tot(U0))
    L = o.get_field(abi.FIELD_L_LOCAL, 1).reshape(desc.K, -1)
    assert L.min() == 0.5 and L.max() <= 1.0
    o.close()


def test_find_alpha_of_equal_states_is_just_above_one():
    """find_alpha (low_order_graph_viscosity.jl:316-340) with ui = uitilde: (alpha - 1) ui
    must have positive density and internal energy, so alpha lands just above 1."""
    from dataclasses import replace

    param, md, bc, desc, U0 = setup(problems.riemann2d, N=2, Kx=4, Ky=4, T=0.2, seed=4)
    pp = replace(param, rhs=p2de.ESLimitedLowOrderPos(low_order_surface_flux=p2de.LaxFriedrichsOnProjectedVal()))
    dts = []
    for prm in (param, pp):
        o = Oracle(S.make_descriptor(prm, md, bc), nthreads=1)
        o.set_Uq(U0)
        dts.append(o.rhs(0.0, 0.2, 1))
        o.close()
    assert dts[1] < dts[0]  # the extra |B| ws / 2 per face shortens the step


def test_reference_semantics_give_low_order_rhs():
    """With the reference's bound destructuring (limiter_utils.jl:66-70) every interior
    subcell face gets factor 0 and rhsU equals the low-order rhsL up to rounding."""
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=6, Ky=6, T=0.1)
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    dt = o.rhs(0.0, 1e-4, 2)
    L = o.get_field(abi.FIELD_L_LOCAL, 2).reshape(desc.K, 2, 20)
    Lx = L[:, 0, :].reshape(desc.K, 4, 5)[:, :, 1:4]
    assert np.all(Lx == 0.0)
    assert relerr(o.get_field(abi.FIELD_RHSU), o.get_field(abi.FIELD_RHSL)) < 1e-12


def test_intended_semantics_keep_high_order_in_smooth_flow():
    # a weak vortex (strength 1): far from vacuum, the positivity bounds never bind
    param, md, bc, desc, U0, *_ = setup(
        problems.isentropic_vortex, N=3, Kx=6, Ky=6, strength=1.0, reference_semantics=False, bound=PositivityBound()
    )
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    o.rhs(0.0, 1e-3, 2)
    assert np.all(o.get_field(abi.FIELD_L_LOCAL, 2) == 1.0)
    assert relerr(o.get_field(abi.FIELD_RHSU), o.get_field(abi.FIELD_RHSH)) < 1e-12
    # the cell entropy bound (subcell.jl:630-744) also acts on rounding-level entropy
    # production, moving a few factors slightly below one
    param, md, bc, desc, U0, *_ = setup(problems.isentropic_vortex, N=3, Kx=6, Ky=6, strength=1.0, reference_semantics=False)
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    o.rhs(0.0, 1e-3, 2)
    assert np.min(o.get_field(abi.FIELD_L_LOCAL, 2)) > 0.99


def test_isentropic_vortex_error_decreases_with_refinement():
    errs = []
    for K in (5, 10):
        param, ic, bcf, exact = problems.isentropic_vortex(N=3, Kx=K, Ky=K, T=0.1, reference_semantics=False)
        md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
        desc = S.make_descriptor(param, md, bcf(param, md))
        o = Oracle(desc, nthreads=2)
        o.set_Uq(S.evaluate_initial_condition(param, md, ic))
        t, n, _ = o.run()
        assert abs(t - 0.1) < 1e-12
        U = o.get_field(abi.FIELD_UQ).reshape(desc.K, -1, 4)
        Ue = problems.primitive_to_conservative(param.equation, exact(param.equation, md.x, md.y, 0.1))
        errs.append(np.abs(U - Ue)[..., 0].max())
    assert errs[1] < 0.5 * errs[0], errs


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("*.npz")))
def test_oracle_matches_golden(name):
    from tests_golden_cases import build

    ref = np.load(GOLDEN / f"{name}.npz")
    param, md, bc, desc, U0, t, dt = build(name)
    np.testing.assert_array_equal(U0.ravel(), ref["U0"])
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    dto = o.rhs(t, dt, 1)
    assert abs(dto - float(ref["dt_out"])) <= 1e-14 * abs(float(ref["dt_out"]))
    for k, f in (("rhsU", abi.FIELD_RHSU), ("rhsL", abi.FIELD_RHSL), ("rhsH", abi.FIELD_RHSH)):
        assert relerr(o.get_field(f), ref[k]) <= 1e-13, k
    np.testing.assert_allclose(o.get_field(abi.FIELD_L_LOCAL), ref["L_local"], atol=1e-13)
    o.step(0.0)
    assert relerr(o.get_field(abi.FIELD_UQ), ref["step_Uq"]) <= 1e-13


# --- CompressibleEulerIdealGas{Dim1} (the Line path) ----------------------------------
def _line(problem, **kw):
    from oracle.binding import Oracle

    param, md, bc, desc, U0 = setup(problem, **kw)
    o = Oracle(desc, nthreads=2)
    o.set_Uq(U0)
    return param, md, desc, U0, o


@pytest.mark.parametrize("basis", ["lobatto", "gauss"])
def test_line_density_wave_conserves_and_converges(basis):
    """The periodic density wave: totals kept to rounding, and the error falls at about
    order N+1 with the element size (positivity bound, inactive on smooth data)."""
    from p2de.types import GaussCollocation, NodewiseScaledExtrapolation, PositivityBound, SubcellLimiter

    kw = dict(approximation_basis=GaussCollocation(), entropyproj_limiter=NodewiseScaledExtrapolation()) \
        if basis == "gauss" else {}
    errs = []
    for K in (8, 16):
        param, md, desc, U0, o = _line(problems.density_wave_1d, N=3, K=K, T=0.1,
                                       rhs_limiter=SubcellLimiter(bound=PositivityBound()), **kw)
        w = np.asarray(o.operator(7))[None, :] * md.geom[:, :1]
        tot0 = (U0 * w[..., None]).sum((0, 1))
        t, n, _ = o.run()
        U = o.get_field(0).reshape(K, -1, 3)
        np.testing.assert_allclose((U * w[..., None]).sum((0, 1)), tot0, rtol=0, atol=1e-13)
        ex = problems.primitive_to_conservative(param.equation, problems.density_wave_1d_exact(None, md.x, t))
        errs.append(np.abs(U - ex).max())
        o.close()
    assert errs[1] < errs[0] / 8, errs


def test_line_free_stream_and_positivity():
    """A constant state stays constant (to rounding) through every bound; Leblanc's shock
    tube keeps positive density and internal energy."""
    from p2de.types import PositivityAndCellEntropyBound, PositivityAndMinEntropyBound, SubcellLimiter, TVDBound

    for bound in (PositivityAndCellEntropyBound(), PositivityAndMinEntropyBound(), TVDBound()):
        param, md, desc, U0, o = _line(problems.density_wave_1d, N=2, K=8, T=0.05,
                                       rhs_limiter=SubcellLimiter(bound=bound))
        U1 = np.broadcast_to(np.array([1.0, 0.5, 2.5]), U0.shape).copy()
        o.set_Uq(U1)
        o.run()
        np.testing.assert_allclose(o.get_field(0).reshape(U0.shape), U1, rtol=0, atol=1e-13)
        o.close()
    param, md, desc, U0, o = _line(problems.leblanc, N=3, K=40, T=0.1)
    o.run()
    U = o.get_field(0).reshape(-1, 3)
    assert U[:, 0].min() > 0 and (U[:, 2] - 0.5 * U[:, 1] ** 2 / U[:, 0]).min() > 0
    o.close()


def test_line_reference_semantics_refused():
    """The reference's Dim1 RHS raises (rhs_utils.jl:18): reference_semantics = 1 is refused
    by the oracle and by the library before any device work."""
    from ctypes import byref, c_void_p

    param, md, bc, desc, U0 = setup(problems.density_wave_1d, N=2, K=4, T=0.1)
    desc.param.reference_semantics = 1
    with pytest.raises(RuntimeError, match="status 2"):
        Oracle(desc)
    lib = abi.load_library()
    h = c_void_p()
    assert lib.p2de_initialize_DG(byref(desc.param), byref(desc.mesh), 0, byref(h)) == 2  # P2DE_ERR_UNSUPPORTED


def test_line_interface_factors_symmetric():
    """Across every element interface the two subcell factors agree after
    symmetrization (mapP pairing of subcell faces 1 and Nq+1), so the limited interface
    flux is one value and the scheme conserves; self-mapped domain ends keep their own."""
    from p2de.types import PositivityAndMinEntropyBound, SubcellLimiter, TVDBound

    for lim in (SubcellLimiter(), SubcellLimiter(bound=TVDBound()), SubcellLimiter(bound=PositivityAndMinEntropyBound())):
        param, md, desc, U0, o = _line(problems.leblanc, N=3, K=20, rhs_limiter=lim)
        o.rhs(param.timestepping_param.t0, 1e-3, 1)
        n1 = param.N + 1
        L = o.get_field(abi.FIELD_L_LOCAL, 1).reshape(desc.K, 2 * n1)
        np.testing.assert_array_equal(L[:-1, n1], L[1:, 0])
        assert L[:, : n1 + 1].min() < 1.0  # the limiter acts at the contact and shock
        o.close()


def test_line_cell_entropy_greedy_acts():
    """The cell-entropy bound's greedy step (enforce_ES_subcell_volume!(::Dim1) with N dvdf
    entries per element) lowers factors below the positivity bound's somewhere on the same
    state: the Shu-Osher data on LGL nodes after 30 steps."""
    from p2de.types import LobattoCollocation, NoEntropyProjectionLimiter, PositivityAndCellEntropyBound
    from p2de.types import PositivityBound, SubcellLimiter

    lgl = dict(approximation_basis=LobattoCollocation(), entropyproj_limiter=NoEntropyProjectionLimiter())
    param, md, desc, U0, o = _line(problems.shu_osher, N=3, K=64, rhs_limiter=SubcellLimiter(bound=PositivityBound()), **lgl)
    t = 0.0
    for _ in range(30):
        t, _ = o.step(t)
    U = o.get_field(abi.FIELD_UQ)
    o.close()
    Ls = []
    for bound in (PositivityBound(), PositivityAndCellEntropyBound()):
        param, md, desc, U0, o = _line(problems.shu_osher, N=3, K=64, rhs_limiter=SubcellLimiter(bound=bound), **lgl)
        o.set_Uq(U)
        o.rhs(t, 1e-3, 1)
        n1 = param.N + 1
        Ls.append(o.get_field(abi.FIELD_L_LOCAL, 1).reshape(desc.K, 2 * n1)[:, : n1 + 1])
        o.close()
    assert np.all(Ls[1] <= Ls[0]) and (Ls[1] < Ls[0]).sum() >= 5
