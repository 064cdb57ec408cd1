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


def test_zerotol_is_read_per_solve_alone_and_in_a_batch():
    """build_op_table drops operator entries at or below ZEROTOL (droptol!, init.jl:147-155,
    312-321), so the operators depend on it: solves with two ZEROTOL values at the same
    degree on one device, alone and as members of one batch, each get their own operators
    (the default value matches the oracle; the batch members equal their solo runs)."""
    from oracle.binding import Oracle

    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=6, Ky=6, T=0.004,
                                    reference_semantics=False, bound=p2de.PositivityBound())
    p2 = replace(param, global_constants=replace(param.global_constants, ZEROTOL=0.02))
    d2 = S.make_descriptor(p2, md, bc)
    solo = {}
    for p, d in ((param, desc), (p2, d2)):
        solo[d.param.ZEROTOL] = alone(p, md, d, U0)[0]
    assert np.max(np.abs(solo[0.02] - solo[5e-16])) > 1e-8 * np.max(np.abs(solo[5e-16]))
    o = Oracle(desc)
    o.set_Uq(U0)
    t = 0.0
    while t < param.timestepping_param.T:
        t, _ = o.step(t)
    ref = o.get_field(abi.FIELD_UQ)
    assert np.max(np.abs(solo[5e-16] - ref)) <= 1e-12 * np.max(np.abs(ref))
    b = Batch(pool_bytes=1 << 28, max_solves=4)
    s1, s2 = b.add(desc, U0), b.add(d2, U0)
    b.run_to_end(chunk=10)
    np.testing.assert_array_equal(b.Uq(s1), solo[5e-16])
    np.testing.assert_array_equal(b.Uq(s2), solo[0.02])
    b.close()


def wide_cases(precision="fp64"):
    """Members of every mode the one-solve path runs on LGL nodes for 2D Euler."""
    from p2de.types import (
        HennemannShockCapture,
        LaxFriedrichsOnProjectedVal,
        PositivityAndMinEntropyBound,
        PositivityAndRelaxedCellEntropyBound,
        PositivityAndRelaxedMinEntropyBound,
        SubcellLimiter,
        TVDAndCellEntropyBound,
        TVDAndMinEntropyBound,
        TVDBound,
        ZhangShuLimiter,
    )

    kw = dict(precision=precision)
    sub = lambda b: dict(rhs_limiter=SubcellLimiter(bound=b))
    cases = [
        setup(problems.riemann2d, N=3, Kx=8, Ky=6, T=0.01, seed=4, **sub(TVDBound()), **kw),
        setup(problems.riemann2d, N=2, Kx=9, Ky=9, T=0.01, seed=5, **sub(TVDAndCellEntropyBound()), **kw),
        setup(problems.isentropic_vortex, N=3, Kx=5, Ky=5, T=0.01, **sub(PositivityAndMinEntropyBound()), **kw),
        setup(problems.isentropic_vortex, N=2, Kx=6, Ky=5, T=0.01, **sub(PositivityAndRelaxedMinEntropyBound()), **kw),
        setup(problems.riemann2d, N=4, Kx=5, Ky=4, T=0.01, seed=6,
              **sub(PositivityAndRelaxedCellEntropyBound(beta=0.5)), reference_semantics=False, **kw),
        setup(problems.double_mach_reflection, N=2, Kx=12, Ky=3, T=0.002, **sub(TVDAndMinEntropyBound()), **kw),
        setup(problems.riemann2d, N=3, Kx=7, Ky=7, T=0.01, seed=7, rhs_limiter=ZhangShuLimiter(), **kw),
        setup(problems.riemann2d, N=2, Kx=8, Ky=8, T=0.01, seed=8,
              rhs_limiter=ZhangShuLimiter(shockcapture=HennemannShockCapture(a=0.5, c=1.8)), **kw),
        setup(problems.kelvin_helmholtz, N=3, Kx=8, Ky=8, T=0.005, **kw),
    ]
    # the projected-value low-order flux (LaxFriedrichsOnProjectedVal) on LGL nodes
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=2, Kx=8, Ky=7, T=0.005, **kw)
    p2 = replace(param, rhs=replace(param.rhs, low_order_surface_flux=LaxFriedrichsOnProjectedVal()))
    cases.append((p2, md, bc, S.make_descriptor(p2, md, bc), U0))
    return cases


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_members_of_every_lgl_mode_equal_their_solo_runs(precision):
    """TVD and min-entropy bounds (the low-only pass and the initial minimum of phi run per
    member inside the batch's step), the relaxed bounds, Zhang-Shu with and without shock
    capture and the projected low-order flux, in one batch with plain members: each member
    runs the kernels it runs alone and ends bitwise equal to its solo run."""
    cases = wide_cases(precision)
    b = Batch(pool_bytes=2 << 30, max_solves=16, precision=precision)
    slots = [b.add(c[3], c[4]) for c in cases]
    b.run_to_end(chunk=7)
    st = b.states()
    for slot, (param, md, bc, desc, U0) in zip(slots, cases):
        U_alone, t_alone, n_alone = alone(param, md, desc, U0)
        assert st[slot, 2] == 1.0 and st[slot, 3] == 0, (slot, st[slot])
        assert st[slot, 0] == t_alone and int(st[slot, 1]) == n_alone
        np.testing.assert_array_equal(b.Uq(slot), U_alone, err_msg=f"member {slot}")
    best = b.autotune()
    assert set(best) == {c[0].N for c in cases}
    b.close()


def test_batch_refuses_gauss_and_kpp_members():
    from p2de.types import GaussCollocation

    param, md, bc, desc, U0 = setup(problems.riemann2d, N=2, Kx=4, Ky=4, T=0.01, seed=1,
                                    approximation_basis=GaussCollocation())
    b = Batch(pool_bytes=1 << 26, max_solves=2)
    with pytest.raises(abi.P2deError) as ei:
        b.add(desc, U0)
    assert ei.value.status == 2
    b.close()
