"""Failure detection through the status word, with the failures made on the host.

The reference stops with a DomainError when a state has a non-positive density or
pressure (log and sqrt of negative values, flux_differencing.jl:49-50,
compressible_Navier_Stokes.jl:48-62). Here the kernels record such states, NaN CFL
candidates and non-positive time steps in a per-solve status word that the host turns
into P2DE_ERR_NOT_POSITIVE (5) or P2DE_ERR_BAD_DT (6); a stepping solve stops at the
next step begin, a served request retires as failed, and nothing else is touched. The
bad inputs are host arrays and parameters: no kernel faults, traps or waits."""
from dataclasses import replace

import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.batch import Server, solve_bytes
from p2de.types import EntropyStable, TimesteppingParameter

from conftest import relerr
from helpers import setup

pytestmark = pytest.mark.gpu

NOT_POSITIVE, BAD_DT = 5, 6


def _bad_states(U0):
    """(name, state) pairs with one node made non-positive or NaN."""
    out = []
    for name, c, val in (("negative density", 0, -1.0), ("negative zero density", 0, -0.0),
                         ("NaN density", 0, float("nan")), ("NaN energy", 3, float("nan"))):
        U = U0.copy()
        U.reshape(-1, 4)[5, c] = val
        out.append((name, U))
    U = U0.copy()  # negative pressure: total energy below the kinetic energy
    row = U.reshape(-1, 4)[7]
    row[3] = 0.25 * (row[1] ** 2 + row[2] ** 2) / row[0]
    out.append(("negative pressure", U))
    return out


def test_rhs_reports_a_nonpositive_state_and_the_handle_stays_usable():
    from oracle.binding import Oracle

    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=6, Ky=6, T=0.1)
    g = S.Solver(param, md, desc)
    for name, U in _bad_states(U0):
        g.set_Uq(U)
        for nstage in (1, 2):
            with pytest.raises(abi.P2deError) as ei:
                S.rhs_bang(None, g, None, p2de.TimeParam(0.0, 0.05, nstage))
            assert ei.value.status == NOT_POSITIVE, (name, nstage, ei.value)
    # a good state clears the status; the result is the oracle's
    g.set_Uq(U0)
    dt = S.rhs_bang(None, g, None, p2de.TimeParam(0.0, 0.05, 1))
    o = Oracle(desc)
    o.set_Uq(U0)
    dto = o.rhs(0.0, 0.05, 1)
    assert abs(dt - dto) <= 1e-13 * dto
    assert relerr(g.get_field(abi.FIELD_RHSU), o.get_field(abi.FIELD_RHSU)) <= 1e-12
    g.close()


def test_rhs_and_step_report_a_bad_time_step():
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=2, Kx=4, Ky=4, T=0.1)
    g = S.Solver(param, md, desc)
    g.set_Uq(U0)
    # stage 1 at t = T: min(CFL dt0, T - t) = 0
    with pytest.raises(abi.P2deError) as ei:
        S.rhs_bang(None, g, None, p2de.TimeParam(0.1, 0.05, 1))
    assert ei.value.status == BAD_DT
    g.close()
    for ts in (TimesteppingParameter(T=0.1, CFL=0.0, dt0=0.1), TimesteppingParameter(T=0.1, CFL=0.5, dt0=float("nan"))):
        p2 = replace(param, timestepping_param=ts)
        d2 = S.make_descriptor(p2, md, bc)
        g = S.Solver(p2, md, d2)
        g.set_Uq(U0)
        with pytest.raises(abi.P2deError) as ei:
            S.ssp33_step(g, 0.0)
        assert ei.value.status == BAD_DT, ts
        np.testing.assert_array_equal(g.get_field(abi.FIELD_UQ), U0.ravel())  # nothing was advanced
        g.close()


def test_stepping_stops_when_an_update_loses_positivity():
    """The unlimited entropy-stable scheme (FluxDiffRHS has no CFL condition of its own, so
    dt = min(CFL dt0, T - t) = T here) loses positivity on a four-quadrant Riemann problem;
    the step that does so reports it and later steps leave the state as it is. The limited
    scheme at CFL 0.5 stays positive at every stage."""
    param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=12, Ky=12, T=0.2, seed=3)
    p_bad = replace(param, rhs=EntropyStable())
    g = S.Solver(p_bad, md, S.make_descriptor(p_bad, md, bc))
    g.set_Uq(U0)
    t, failed = 0.0, None
    for i in range(30):
        try:
            t, _ = S.ssp33_step(g, t)
        except abi.P2deError as e:
            failed = (i, e.status)
            break
    assert failed is not None and failed[1] == NOT_POSITIVE, failed
    U_stop = g.get_field(abi.FIELD_UQ)
    with pytest.raises(abi.P2deError) as ei:
        S.ssp33_step(g, t)
    assert ei.value.status == NOT_POSITIVE
    np.testing.assert_array_equal(g.get_field(abi.FIELD_UQ), U_stop)
    g.close()
    g = S.Solver(param, md, desc)
    g.set_Uq(U0)
    t = 0.0
    for _ in range(5):
        t, _ = S.ssp33_step(g, t)
    mins = np.zeros(6)
    g._check(g.lib.p2de_stage_minima(g.handle, abi.dptr(mins)))
    assert np.all(mins > 0)
    g.close()


def test_server_retires_a_failed_request_and_finishes_the_others():
    from test_gpu_batch import alone, mix_cases

    cases = mix_cases()[:4]
    param, md, bc, desc, U0 = cases[1]
    U_bad = U0.copy()
    U_bad.reshape(-1, 4)[3, 0] = -1.0
    budget = sum(solve_bytes(c[3]) for c in cases) * 2
    sv = Server(hbm_budget_bytes=budget, max_active=8, steps_per_tick=4)
    ids = [sv.submit(c[3], c[4]) for c in cases[:2]]
    bad = sv.submit(desc, U_bad)
    ids += [sv.submit(c[3], c[4]) for c in cases[2:]]
    assert sv.wait(bad, timeout_s=120) == Server.FAILED
    for rid in ids:
        assert sv.wait(rid, timeout_s=120) == Server.DONE
    for rid, (p, m, b, d, U) in zip(ids, cases):
        U_alone, t_alone, n_alone = alone(p, m, d, U)
        info = sv.poll(rid)
        assert info.t_final == t_alone and info.steps == n_alone
        np.testing.assert_array_equal(sv.result(rid), U_alone)
    st = sv.stats()
    assert st["failed"] == 1 and st["completed"] == len(cases) and st["active"] == 0
    sv.close()
