"""Host-side logic: the StartUpDG-convention mesh, boundary classification, the
lowering of Param's dispatch types, and the replica path of bench.py on two gloo
ranks (CPU only)."""
import os
import socket

import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.types import (
    EntropyStable,
    GaussCollocation,
    HennemannShockCapture,
    LowOrderPositivity,
    NodewiseScaledExtrapolation,
    NoRHSLimiter,
    PositivityAndRelaxedCellEntropyBound,
    PositivityBound,
    SubcellLimiter,
    ZhangShuLimiter,
)


@pytest.mark.parametrize("N,Kx,Ky", [(1, 3, 2), (3, 4, 5), (5, 2, 2)])
def test_periodic_mapP_is_an_involution_matching_coordinates(N, Kx, Ky):
    md = p2de.make_periodic(p2de.uniform_mesh(N, Kx, Ky, (0.0, 0.0), (2.0, 3.0)))
    mP = md.mapP.ravel() - 1
    assert np.all(mP[mP] == np.arange(mP.size))
    assert md.mapB.size == 0
    xf, yf = md.xf.ravel(), md.yf.ravel()
    dx = np.abs(xf - xf[mP])
    dy = np.abs(yf - yf[mP])
    # partners coincide, or differ by a period across the wrap
    assert np.all((dx < 1e-12) | (np.abs(dx - 2.0) < 1e-12))
    assert np.all((dy < 1e-12) | (np.abs(dy - 3.0) < 1e-12))


@pytest.mark.parametrize("N,Kx,Ky", [(1, 3, 2), (3, 4, 5), (4, 3, 3)])
def test_face_order_matches_the_reference_subcell_index_maps(N, Kx, Ky):
    """The face-node order and the mapP partners that the reference's limiter code takes for
    granted, independently of how mesh.py builds them: subcell_face_idx_to_quad_face_index_x/y
    and subcell_index_P_x/y (src/dg/limiter/limiter_utils.jl:97-181) read face node
    f = sj (r = -1), N1D + sj (r = +1), 2 N1D + si (s = -1), 3 N1D + si (s = +1) with
    volume node q = si + N1D sj (0-based), and take an r-face's partner on the neighbour's
    r-faces at the same sj and an s-face's partner on its s-faces at the same si."""
    md = p2de.make_periodic(p2de.uniform_mesh(N, Kx, Ky, (0.0, 0.0), (2.0, 1.0)))
    n = N + 1
    x, y, xf, yf = md.x, md.y, md.xf, md.yf
    # volume nodes: r (x) fastest, then s (y)
    X = x.reshape(-1, n, n)
    Y = y.reshape(-1, n, n)
    assert np.all(np.diff(X, axis=2) > 0) and np.all(np.abs(np.diff(X, axis=1)) < 1e-14)
    assert np.all(np.diff(Y, axis=1) > 0) and np.all(np.abs(np.diff(Y, axis=2)) < 1e-14)
    for f in range(4 * n):
        side, t = divmod(f, n)
        si, sj = ((0, t), (N, t), (t, 0), (t, N))[side]
        q = si + n * sj
        assert np.allclose(xf[:, f], x[:, q], atol=1e-14) and np.allclose(yf[:, f], y[:, q], atol=1e-14), f
    mP = md.mapP - 1
    for k in range(md.num_elements):
        for f in range(4 * n):
            kP, iP = divmod(int(mP[k, f]), 4 * n)
            side, t = divmod(f, n)
            sideP, tP = divmod(iP, n)
            assert tP == t, (k, f, iP)
            assert sideP == {0: 1, 1: 0, 2: 3, 3: 2}[side], (k, f, iP)
            assert kP != k or (Kx == 1 and side < 2) or (Ky == 1 and side >= 2)


def test_boundary_sides_of_an_open_mesh():
    N, Kx, Ky = 2, 4, 3
    md = p2de.uniform_mesh(N, Kx, Ky)
    n = N + 1
    assert md.mapB.size == 2 * n * (Kx + Ky)
    for side, x_or_y, val in (("left", "xf", 0.0), ("right", "xf", 1.0), ("bottom", "yf", 0.0), ("top", "yf", 1.0)):
        idx = md.sides[side] - 1
        assert np.allclose(getattr(md, x_or_y).ravel()[idx], val)
    mP = md.mapP.ravel() - 1
    inner = np.setdiff1d(np.arange(mP.size), md.mapB - 1)
    assert np.all(mP[mP[inner]] == inner)


def test_double_mach_boundary_classification():
    param, ic, bcf = problems.double_mach_reflection(N=3, Kx=24, Ky=6)
    md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
    bc = bcf(param, md)
    xf = md.xf.ravel()
    n = 4
    assert len(bc.mapO) == 6 * n and len(bc.mapS) == 24 * n
    assert np.all(xf[bc.mapW - 1] >= 1 / 6)
    assert len(bc.mapI) == 6 * n + np.sum(xf[md.sides["bottom"] - 1] < 1 / 6)
    assert len(np.intersect1d(bc.mapI, bc.mapW)) == 0
    U0 = S.evaluate_initial_condition(param, md, ic)
    assert set(np.unique(U0[..., 0])) == {1.4, 8.0}


def test_lowering_rejects_what_is_not_built():
    from dataclasses import replace

    param, ic, bcf = problems.kelvin_helmholtz(N=3, Kx=2, Ky=2)
    K = 4
    assert S.lower_param(param, K).rhs_type == 0
    assert S.lower_param(replace(param, rhs=LowOrderPositivity()), K).rhs_type == 1
    assert S.lower_param(replace(param, rhs=EntropyStable()), K).rhs_type == 2
    assert S.lower_param(replace(param, approximation_basis=GaussCollocation()), K).approximation_basis == abi.BASIS_GAUSS
    g = S.lower_param(replace(param, approximation_basis=GaussCollocation(), entropyproj_limiter=NodewiseScaledExtrapolation(),
                              rhs_limiter=SubcellLimiter(bound=PositivityBound())), K)
    assert g.approximation_basis == abi.BASIS_GAUSS
    assert g.entropyproj_limiter == abi.ENTROPYPROJ_NODEWISE_SCALED_EXTRAPOLATION
    relaxed = S.lower_param(replace(param, rhs_limiter=SubcellLimiter(bound=PositivityAndRelaxedCellEntropyBound(0.25))), K)
    assert relaxed.bound_type == abi.BOUND_POSITIVITY_AND_RELAXED_CELL_ENTROPY and relaxed.bound_beta == 0.25
    zs = S.lower_param(replace(param, rhs_limiter=ZhangShuLimiter(shockcapture=HennemannShockCapture())), K)
    assert zs.rhs_limiter == abi.LIMITER_ZHANG_SHU and zs.shock_capture == 1
    with pytest.raises(S.UnsupportedMethod):
        S.lower_param(replace(param, rhs_limiter=NoRHSLimiter()), K)
    with pytest.raises(S.UnsupportedMethod):
        S.lower_param(replace(param, precision="bf16"), K)
    assert S.lower_param(replace(param, precision="mixed"), K).precision == 1


def test_initial_conditions_are_seeded():
    p1, ic1, _ = problems.kelvin_helmholtz(N=2, Kx=4, Ky=4, seed=0)
    md = p2de.uniform_mesh(2, 4, 4)
    a = S.evaluate_initial_condition(p1, md, ic1)
    b = S.evaluate_initial_condition(p1, md, ic1)
    np.testing.assert_array_equal(a, b)
    p2, ic2, _ = problems.kelvin_helmholtz(N=2, Kx=4, Ky=4, seed=1)
    assert not np.array_equal(a, S.evaluate_initial_condition(p2, md, ic2))
    s = problems.riemann_quadrant_states(3)
    assert s.shape == (4, 4) and np.all(s[:, 0] >= 0.1) and np.all(s[:, 3] >= 0.02)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_rank(rank, world, port, out):
    """One replica: an independent solve per rank (different seed), timing reduced by
    MAX and units by SUM, as bench.py does for --gpus N."""
    import sys
    import time
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root / "p2de.jl_gb300"))
    sys.path.insert(0, str(root))
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import p2de as P
    from p2de import problems as pr
    from p2de import solver as SS
    from oracle.binding import Oracle

    param, ic, bcf = pr.riemann2d(N=2, Kx=4, Ky=4, seed=10 + rank)
    md = P.uniform_mesh(param.N, *param.K, param.xL, param.xR)
    desc = SS.make_descriptor(param, md, bcf(param, md))
    o = Oracle(desc, nthreads=1)
    o.set_Uq(SS.evaluate_initial_condition(param, md, ic))
    dist.barrier()
    t0 = time.perf_counter()
    t = 0.0
    for _ in range(2):
        t, _ = o.step(t)
    el = torch.tensor([time.perf_counter() - t0], dtype=torch.float64)
    units = torch.tensor([float(desc.K * desc.Nq * 3 * 2)], dtype=torch.float64)
    dist.all_reduce(el, op=dist.ReduceOp.MAX)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    rho_min = torch.tensor([o.get_field(0).reshape(-1, 4)[:, 0].min()], dtype=torch.float64)
    gathered = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(gathered, rho_min)
    if rank == 0:
        out.put((el.item(), units.item(), [g.item() for g in gathered]))
    dist.destroy_process_group()


def test_replicas_on_two_gloo_ranks():
    import torch.multiprocessing as mp

    from oracle import binding

    binding.build()  # once, here: the two ranks must not rebuild it concurrently
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    el, units, rho = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert units == 2 * 16 * 9 * 3 * 2
    assert el > 0
    assert len(rho) == 2 and rho[0] != rho[1] and min(rho) > 0
