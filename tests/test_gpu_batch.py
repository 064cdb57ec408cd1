"""Batched solves and the continuous-batching server: each solve's result in a batch
or in the served mix equals its result alone (bitwise: the element arithmetic is
shared), every solve stops at its own final time, admission respects the HBM budget."""
from dataclasses import replace

import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.batch import Batch, Server, solve_bytes

from helpers import setup

pytestmark = pytest.mark.gpu


def mix_cases(precision="fp64"):
    kw = dict(precision=precision)
    return [
        setup(problems.kelvin_helmholtz, N=3, Kx=12, Ky=10, T=0.01, **kw),
        setup(problems.riemann2d, N=2, Kx=16, Ky=16, T=0.02, seed=4, **kw),
        setup(problems.double_mach_reflection, N=3, Kx=16, Ky=4, T=0.003, **kw),
        setup(problems.riemann2d, N=4, Kx=7, Ky=9, T=0.015, seed=9, **kw),
        setup(problems.kelvin_helmholtz, N=1, Kx=20, Ky=20, T=0.01, **kw),
        setup(problems.riemann2d, N=5, Kx=4, Ky=4, T=0.01, seed=2, **kw),
    ]


def alone(param, md, desc, U0):
    g = S.Solver(param, md, desc)
    g.set_Uq(U0)
    t, n, dt = c_run(g)
    U = g.get_field(abi.FIELD_UQ)
    g.close()
    return U, t, n


def c_run(g):
    from ctypes import byref, c_double, c_int64

    t, n, dt = c_double(), c_int64(), c_double()
    g._check(g.lib.p2de_ssp33(g.handle, byref(t), byref(n), byref(dt)))
    return t.value, n.value, dt.value


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-acc64"])
def test_batch_members_equal_their_solo_runs(precision):
    cases = mix_cases(precision)
    b = Batch(pool_bytes=2 << 30, max_solves=16, precision=precision)
    slots = [b.add(c[3], c[4]) for c in cases]
    b.run_to_end(chunk=20)
    st = b.states()
    for slot, (param, md, bc, desc, U0) in zip(slots, cases):
        U_alone, t_alone, n_alone = alone(param, md, desc, U0)
        assert st[slot, 2] == 1.0 and st[slot, 3] == 0
        assert st[slot, 0] == t_alone and abs(t_alone - param.timestepping_param.T) < 1e-12
        assert int(st[slot, 1]) == n_alone
        np.testing.assert_array_equal(b.Uq(slot), U_alone)
    b.close()


def test_batch_admission_by_budget_and_reuse():
    cases = mix_cases()
    sizes = [solve_bytes(c[3]) for c in cases]
    pool = sizes[0] + sizes[1] + 4096
    b = Batch(pool_bytes=pool, max_solves=8)
    s0 = b.add(cases[0][3], cases[0][4])
    s1 = b.add(cases[1][3], cases[1][4])
    with pytest.raises(abi.P2deError) as ei:
        b.add(cases[2][3], cases[2][4])
    assert ei.value.status == 8
    b.remove(s0)
    j = min(range(2, len(cases)), key=lambda i: sizes[i])  # fits the freed block
    assert sizes[j] <= sizes[0]
    s2 = b.add(cases[j][3], cases[j][4])
    b.run_to_end(chunk=20)
    U_alone, _, _ = alone(cases[j][0], cases[j][1], cases[j][3], cases[j][4])
    np.testing.assert_array_equal(b.Uq(s2), U_alone)
    used, cap = b.memory()
    assert used <= cap
    b.close()


def test_server_serves_a_mix_with_results_equal_alone():
    cases = mix_cases()
    budget = sum(solve_bytes(c[3]) for c in cases[:3]) + (1 << 20)
    sv = Server(hbm_budget_bytes=budget, max_active=8, steps_per_tick=4)
    ids = [sv.submit(c[3], c[4]) for c in cases]
    for rid in ids:
        assert sv.wait(rid, timeout_s=120) == Server.DONE
    infos = [sv.poll(rid) for rid in ids]
    assert all(i.latency_s > 0 for i in infos)
    for rid, (param, md, bc, desc, U0), info in zip(ids, cases, infos):
        U_alone, t_alone, n_alone = alone(param, md, desc, U0)
        assert info.t_final == t_alone and info.steps == n_alone
        np.testing.assert_array_equal(sv.result(rid), U_alone)
    st = sv.stats()
    assert st["completed"] == len(cases) and st["failed"] == 0 and st["active"] == 0
    sv.close()


def test_server_rejects_a_request_larger_than_the_budget():
    param, md, bc, desc, U0 = mix_cases()[0]
    sv = Server(hbm_budget_bytes=solve_bytes(desc) // 2, max_active=2)
    with pytest.raises(abi.P2deError) as ei:
        sv.submit(desc, U0)
    assert ei.value.status == 8
    sv.close()


def test_batch_member_with_shock_capture_equals_alone():
    """Members with HennemannShockCapture keep their per-solve blending constants in the
    batch; the result equals the solve alone."""
    from p2de.types import HennemannShockCapture, PositivityAndCellEntropyBound, SubcellLimiter

    param, md, bc, desc, U0 = setup(problems.riemann2d, N=3, Kx=10, Ky=8, T=0.01, seed=12)
    ps = replace(param, rhs_limiter=SubcellLimiter(bound=PositivityAndCellEntropyBound(),
                                                   shockcapture=HennemannShockCapture(a=0.4, c=1.7)))
    ds = S.make_descriptor(ps, md, bc)
    b = Batch(pool_bytes=1 << 30, max_solves=4)
    s0 = b.add(ds, U0)
    s1 = b.add(desc, U0)  # the same problem without shock capture
    b.run_to_end(chunk=10)
    U_sc, _, _ = alone(ps, md, ds, U0)
    U_no, _, _ = alone(param, md, desc, U0)
    np.testing.assert_array_equal(b.Uq(s0), U_sc)
    np.testing.assert_array_equal(b.Uq(s1), U_no)
    assert np.abs(U_sc - U_no).max() > 0  # the capture changed the solution
    b.close()
