"""Elements per block, thread layouts of the pair phases and the autotuner: the launch
shape does not change any result (each element's arithmetic is the same at every value
and in every layout, and the only cross-element reductions are exact minima), so runs at
any elements-per-block, in either layout, and runs after autotuning, are bitwise equal to
runs at the default."""
from ctypes import byref, c_double, c_int64

import numpy as np
import pytest

from p2de import abi, problems
from p2de import solver as S
from p2de.batch import Batch

from helpers import setup
from test_gpu_batch import alone, mix_cases

pytestmark = pytest.mark.gpu


def run_steps(param, md, desc, U0, nsteps, epb=None, tune=False, layout=None, threads=None):
    g = S.Solver(param, md, desc)
    g.set_Uq(U0)
    if threads is not None:
        g.set_threads_per_block(threads)
        assert g.threads_per_block() == threads
    if epb is not None:
        g.set_elements_per_block(epb)
    if layout is not None:
        g.set_layout(layout)
        assert g.layout() == layout
    if tune:
        best, ms = g.autotune()
        assert 1 <= best <= g.elements_per_block()[1] and ms > 0
        assert g.elements_per_block()[0] == best
        assert g.layout() in (abi.LAYOUT_FLAT, abi.LAYOUT_LINES_PER_WARP)
        # tuning leaves the state alone
        np.testing.assert_array_equal(g.get_field(abi.FIELD_UQ), np.ravel(U0))
    t, n = c_double(0.0), c_int64()
    g._check(g.lib.p2de_ssp33_advance(g.handle, nsteps, byref(t), byref(n)))
    U = g.get_field(abi.FIELD_UQ)
    g.close()
    return U, t.value


@pytest.mark.parametrize(
    "problem,N,kw",
    [
        (problems.kelvin_helmholtz, 1, dict(Kx=12, Ky=10)),
        (problems.double_mach_reflection, 2, dict(Kx=16, Ky=4)),
        (problems.kelvin_helmholtz, 3, dict(Kx=9, Ky=7)),
        (problems.riemann2d, 4, dict(Kx=6, Ky=5, seed=3)),
        (problems.riemann2d, 5, dict(Kx=5, Ky=3, seed=8)),
    ],
)
def test_elements_per_block_does_not_change_results(problem, N, kw):
    param, md, bc, desc, U0 = setup(problem, N=N, T=0.2, **kw)
    U_ref, t_ref = run_steps(param, md, desc, U0, 4)
    g = S.Solver(param, md, desc)
    edef, emax = g.elements_per_block()
    g.close()
    assert 1 <= edef <= emax
    for e in sorted({1, 3, max(1, edef // 2), emax}):
        U, t = run_steps(param, md, desc, U0, 4, epb=e)
        assert t == t_ref
        np.testing.assert_array_equal(U, U_ref, err_msg=f"epb={e}")
    U, t = run_steps(param, md, desc, U0, 4, tune=True)
    assert t == t_ref
    np.testing.assert_array_equal(U, U_ref)


def test_mixed_precision_elements_per_block():
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=10, Ky=10, T=0.2, precision="mixed")
    U_ref, t_ref = run_steps(param, md, desc, U0, 3)
    for e in (1, 5):
        U, t = run_steps(param, md, desc, U0, 3, epb=e)
        assert t == t_ref
        np.testing.assert_array_equal(U, U_ref)


def test_elements_per_block_range_is_checked():
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=2, Kx=4, Ky=4, T=0.1)
    g = S.Solver(param, md, desc)
    edef, emax = g.elements_per_block()
    for bad in (0, -1, emax + 1):
        with pytest.raises(abi.P2deError) as ei:
            g.set_elements_per_block(bad)
        assert ei.value.status == 1  # P2DE_ERR_INVALID_ARGUMENT
    assert g.elements_per_block()[0] == edef
    g.close()


@pytest.mark.parametrize("how", ["set", "autotune"])
def test_batch_elements_per_block_keeps_members_equal_alone(how):
    cases = mix_cases()
    b = Batch(pool_bytes=2 << 30, max_solves=16)
    slots = [b.add(c[3], c[4]) for c in cases]
    if how == "set":
        for N, e in {1: 3, 2: 1, 3: 7, 4: 2, 5: 1}.items():
            b.set_elements_per_block(N, e)
            assert b.elements_per_block(N)[0] == e
    else:
        before = [b.Uq(s) for s in slots]
        best = b.autotune()
        assert set(best) == {c[0].N for c in cases}
        for N, e in best.items():
            assert 1 <= e <= b.elements_per_block(N)[1]
        for s, U in zip(slots, before):
            np.testing.assert_array_equal(b.Uq(s), U)
    b.run_to_end(chunk=20)
    st = b.states()
    for slot, (param, md, bc, desc, U0) in zip(slots, cases):
        U_alone, t_alone, n_alone = alone(param, md, desc, U0)
        assert st[slot, 2] == 1.0 and st[slot, 3] == 0
        assert st[slot, 0] == t_alone and int(st[slot, 1]) == n_alone
        np.testing.assert_array_equal(b.Uq(slot), U_alone)
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed-acc64"])
@pytest.mark.parametrize(
    "problem,N,kw",
    [
        (problems.kelvin_helmholtz, 1, dict(Kx=12, Ky=10)),
        (problems.double_mach_reflection, 2, dict(Kx=16, Ky=4)),
        (problems.kelvin_helmholtz, 3, dict(Kx=9, Ky=7)),
        (problems.riemann2d, 4, dict(Kx=6, Ky=5, seed=3)),
        (problems.riemann2d, 5, dict(Kx=5, Ky=3, seed=8)),
    ],
)
def test_lines_per_warp_layout_gives_the_same_bits(problem, N, kw, precision):
    """The whole-lines-per-warp layout of the pair phases against the flat layout, at the
    default and at extreme elements per block (partial warps of lines at the block's end)."""
    param, md, bc, desc, U0 = setup(problem, N=N, T=0.2, precision=precision, **kw)
    U_ref, t_ref = run_steps(param, md, desc, U0, 4, layout=abi.LAYOUT_FLAT)
    g = S.Solver(param, md, desc)
    edef, emax = g.elements_per_block()
    g.close()
    for e in sorted({1, edef, emax}):
        U, t = run_steps(param, md, desc, U0, 4, epb=e, layout=abi.LAYOUT_LINES_PER_WARP)
        assert t == t_ref
        np.testing.assert_array_equal(U, U_ref, err_msg=f"epb={e}")


def test_lines_per_warp_layout_on_rotated_elements_runs_flat():
    """Elements that are not axis-aligned have pair terms on both axes; the layout setting
    leaves them on the flat loops, with the same result."""
    import p2de

    param, ic, bcf = problems.isentropic_vortex(N=3, Kx=5, Ky=5, reference_semantics=False)[:3]
    md = p2de.mesh.rotated(p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR), 0.3)
    bc = bcf(param, md)
    desc = S.make_descriptor(param, md, bc)
    U0 = S.evaluate_initial_condition(param, md, ic)
    U_ref, _ = run_steps(param, md, desc, U0, 3, layout=abi.LAYOUT_FLAT)
    U, _ = run_steps(param, md, desc, U0, 3, layout=abi.LAYOUT_LINES_PER_WARP)
    np.testing.assert_array_equal(U, U_ref)


def test_layout_value_is_checked():
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=2, Kx=4, Ky=4, T=0.1)
    g = S.Solver(param, md, desc)
    for bad in (-1, 2):
        with pytest.raises(abi.P2deError) as ei:
            g.set_layout(bad)
        assert ei.value.status == 1
    assert g.layout() == abi.LAYOUT_FLAT
    g.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_layout_keeps_members_equal_alone(precision):
    cases = mix_cases(precision)
    b = Batch(pool_bytes=2 << 30, max_solves=16, precision=precision)
    slots = [b.add(c[3], c[4]) for c in cases]
    for N in {c[0].N for c in cases}:
        b.set_layout(N, abi.LAYOUT_LINES_PER_WARP)
        assert b.layout(N) == abi.LAYOUT_LINES_PER_WARP
    b.run_to_end(chunk=20)
    for slot, (param, md, bc, desc, U0) in zip(slots, cases):
        U_alone, t_alone, n_alone = alone(param, md, desc, U0)
        np.testing.assert_array_equal(b.Uq(slot), U_alone)
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize(
    "problem,N,kw",
    [
        (problems.kelvin_helmholtz, 1, dict(Kx=12, Ky=10)),
        (problems.double_mach_reflection, 3, dict(Kx=16, Ky=4)),
        (problems.riemann2d, 5, dict(Kx=5, Ky=3, seed=8)),
    ],
)
def test_threads_per_block_gives_the_same_bits(problem, N, kw, precision):
    """Stage kernel A with 64 threads per block (every phase loops over its items with the
    block's size) against the default 128, in both layouts."""
    param, md, bc, desc, U0 = setup(problem, N=N, T=0.2, precision=precision, **kw)
    U_ref, t_ref = run_steps(param, md, desc, U0, 4)
    for layout in (abi.LAYOUT_FLAT, abi.LAYOUT_LINES_PER_WARP):
        U, t = run_steps(param, md, desc, U0, 4, threads=64, layout=layout)
        assert t == t_ref
        np.testing.assert_array_equal(U, U_ref, err_msg=f"layout {layout}")
