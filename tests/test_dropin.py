"""The drop-in boundary as the reference's callers use it: SSP33! (SSPRK33.jl:25-41)
calls rhs!(state, solver, state_param, time_param) three times per step and rewrites
state.preallocation.Uq on the host between the calls. HostState + rhs_bang reproduce that
contract over the C ABI; SSP33_host_loop restates the loop over host arrays.

CPU: the loop, driven by the oracle's right-hand side, equals the oracle's own SSP-RK3
step bit for bit (it is the same arithmetic). GPU: the loop driven by rhs_bang through
the C ABI matches the oracle at 1e-12 per step for the three rhs! dispatch types and both
limiter semantics, and rhs_bang reads the host Uq it is given, not the device's copy."""
from dataclasses import replace

import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.types import EntropyStable, LowOrderPositivity

from conftest import relerr
from helpers import setup


class _OracleSolve:
    """What SSP33_host_loop reads of a solver, over an oracle solve."""

    def __init__(self, param, desc):
        from oracle.binding import Oracle

        self.param, self.desc = param, desc
        self.o = Oracle(desc)
        self.K, self.Nq, self.N1D = desc.K, desc.Nq, desc.N + 1


def _oracle_rhs(state, solver, state_param, tp):
    pre = state.preallocation
    solver.o.set_Uq(pre.Uq)
    dt = solver.o.rhs(tp.t, tp.dt, tp.nstage)
    pre.rhsU[...] = solver.o.get_field(abi.FIELD_RHSU).reshape(pre.rhsU.shape)
    return dt


def test_host_loop_restates_ssp33_bit_for_bit_with_the_oracle():
    from oracle.binding import Oracle

    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=6, Ky=6, T=0.1)
    fake = _OracleSolve(param, desc)
    st = S.HostState(fake, U0)
    ref = Oracle(desc)
    ref.set_Uq(U0)
    t_ref = 0.0
    t, dts = S.SSP33_host_loop(st, fake, S.StateParam(bc), nsteps=3, rhs=_oracle_rhs)
    for _ in range(3):
        t_ref, _ = ref.step(t_ref)
    assert t == t_ref and len(dts) == 3
    np.testing.assert_array_equal(st.preallocation.Uq.ravel(), ref.get_field(abi.FIELD_UQ))


RHS_CASES = [
    ("limited-ref", {}),
    ("limited-intended-positivity", dict(reference_semantics=False, bound=p2de.PositivityBound())),
    ("low-order", "low"),
    ("entropy-stable", "es"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw", RHS_CASES, ids=[c[0] for c in RHS_CASES])
def test_host_loop_through_rhs_bang_matches_the_oracle(name, kw):
    from oracle.binding import Oracle

    extra = kw if isinstance(kw, dict) else {}
    if kw == "es":  # the unlimited scheme on smooth data
        param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=8, Ky=8, T=0.05)
    else:
        param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=8, Ky=8, T=0.05, seed=5, **extra)
    if kw == "low":
        param = replace(param, rhs=LowOrderPositivity())
    elif kw == "es":
        param = replace(param, rhs=EntropyStable(), timestepping_param=replace(param.timestepping_param, dt0=1e-3))
    desc = S.make_descriptor(param, md, bc)
    g = S.Solver(param, md, desc)
    st = S.HostState(g, U0)
    o = Oracle(desc)
    o.set_Uq(U0)
    t, t_o = 0.0, 0.0
    for step in range(3):
        t, dts = S.SSP33_host_loop(st, g, S.StateParam(bc), nsteps=1, t_start=t)
        t_o, dt_o = o.step(t_o)
        assert abs(dts[0] - dt_o) <= 1e-13 * dt_o, (step, dts[0], dt_o)
        assert abs(t - t_o) <= 1e-13 * t_o
        e = relerr(st.preallocation.Uq, o.get_field(abi.FIELD_UQ))
        assert e <= 1e-12, (name, step, e)
    # rhs_bang uses the Uq of the state it is given: a different host state, same handle
    st0 = S.HostState(g, U0)
    dt = S.rhs_bang(st0, g, None, p2de.TimeParam(0.0, 0.01, 1))
    o.set_Uq(U0)
    dto = o.rhs(0.0, 0.01, 1)
    assert abs(dt - dto) <= 1e-13 * abs(dto)
    assert relerr(st0.preallocation.rhsU, o.get_field(abi.FIELD_RHSU)) <= 1e-12
    g.close()
