"""Device diagnostics against their numpy restatements: check_conservation
(src/dg/utils.jl:1-12) and calculate_error (src/dg/postprocess.jl:1-46)."""
import numpy as np
import pytest

from p2de import abi, problems
from p2de import solver as S
from p2de.mesh import gll_rule

from helpers import setup

pytestmark = pytest.mark.gpu


def weights(solver):
    _, w = gll_rule(solver.N)
    n = solver.N1D
    wq = w[np.tile(np.arange(n), n)] * w[np.repeat(np.arange(n), n)]
    return solver.md.geom[:, 0:1] * wq[None, :]


def conservation_np(U, W):
    return np.einsum("ki,kic->c", W, U.reshape(W.shape[0], W.shape[1], 4))


def close_sums(a, U, W):
    # sums of n terms in different orders agree to ~n eps times the sum of the magnitudes
    scale = np.einsum("ki,kic->c", W, np.abs(U.reshape(W.shape[0], W.shape[1], 4)))
    assert np.all(np.abs(a - conservation_np(U, W)) <= 1e-12 * scale), (a, conservation_np(U, W))


def errors_np(U, Ue, W):
    U = U.reshape(Ue.shape)
    e = np.abs(Ue - U)
    w = W[..., None]
    L1e, L2e, Linfe = (w * e).sum((0, 1)), (w * e**2).sum((0, 1)), e.max((0, 1))
    L1x, L2x, Linfx = (w * np.abs(Ue)).sum((0, 1)), (w * Ue**2).sum((0, 1)), np.abs(Ue).max((0, 1))
    m = Linfx > 1e-14
    return ((L1e[m] / L1x[m]).sum(), (np.sqrt(L2e[m]) / np.sqrt(L2x[m])).sum(), (Linfe[m] / Linfx[m]).sum())


def test_conservation_matches_and_is_conserved():
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=16, Ky=12, T=0.2)
    g = S.Solver(param, md, desc)
    g.set_Uq(U0)
    W = weights(g)
    t0 = S.conservation_totals(g)
    close_sums(t0, U0, W)
    t = 0.0
    for _ in range(5):
        t, _ = S.ssp33_step(g, t)
    t1 = S.conservation_totals(g)
    U1 = g.get_field(abi.FIELD_UQ)
    close_sums(t1, U1, W)
    scale = np.einsum("ki,kic->c", W, np.abs(U1.reshape(W.shape[0], W.shape[1], 4)))
    assert np.all(np.abs(t1 - t0) <= 1e-12 * scale)  # periodic: conserved
    assert S.check_conservation(S.State(g), g) == S.check_conservation(S.State(g), g)  # deterministic
    g.close()


def test_calculate_error_matches():
    param, ic, bcf, exact = problems.isentropic_vortex(N=3, Kx=8, Ky=8, T=0.05, strength=1.0)
    import p2de

    md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
    desc = S.make_descriptor(param, md, bcf(param, md))
    U0 = S.evaluate_initial_condition(param, md, ic)
    g = S.Solver(param, md, desc)
    g.set_Uq(U0)
    S.SSP33_bang(S.State(g), g, None, snapshots=False)
    err = S.calculate_error(S.State(g), g, exact)
    Ue = S.exact_nodal_values(g, exact, param.timestepping_param.T)
    ref = errors_np(g.get_field(abi.FIELD_UQ), Ue, weights(g))
    np.testing.assert_allclose([err.L1err, err.L2err, err.Linferr], ref, rtol=1e-12)
    assert all(np.isfinite([err.L1err, err.L2err, err.Linferr])) and err.L1err > 0
    g.close()
