"""p2de_rhs_noalloc: the right-hand side for callers that cannot allocate device memory
(a process whose HBM is reserved by its own pool allocator, or an application that
allocates device memory only at start-up). The test owns every device buffer (allocated
here with torch); the entry point runs with only its static scratch array. Its output
must equal the regular entry point's (p2de_rhs on a solver handle) within the parity
tolerance, and the oracle's, on consecutive calls, which also checks that the shared
scratch carries nothing over from one call to the next; the device's free memory must
not change across those calls. This file is collected last so that a run that stops at
its first failure has already run every other test."""
import ctypes
from ctypes import byref, c_double, c_int64
from dataclasses import replace

import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S
from p2de.noalloc import device_mesh_arrays

from conftest import relerr
from helpers import setup

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _device_mesh(torch, arrs, bc):
    t = {
        "geom": torch.from_numpy(arrs["geom"]).cuda(),
        "nbr": torch.from_numpy(arrs["nbr"]).cuda(),
        "bc": torch.from_numpy(arrs["bc"]).cuda(),
        "bcidx": torch.from_numpy(arrs["bcidx"]).cuda(),
        "Ival": torch.from_numpy(arrs["Ival"]).cuda(),
        "xyS": torch.from_numpy(arrs["xyS"]).cuda(),
    }
    m = abi.P2deDeviceMesh()
    for k in ("geom", "nbr", "bc", "bcidx", "Ival", "xyS"):
        setattr(m, k, t[k].data_ptr())
    m.nI, m.nS = arrs["nI"], arrs["nS"]
    m.shock_x0, m.shock_inv_slope, m.shock_speed = bc.shock_x0, bc.shock_inv_slope, bc.shock_speed
    for c in range(4):
        m.shock_post[c] = bc.shock_post[c]
        m.shock_pre[c] = bc.shock_pre[c]
    m.axis_aligned = arrs["axis_aligned"]
    return m, t


def _regular_rhs(param, md, desc, U0, t, dt, nstage):
    g = S.Solver(param, md, desc)
    g.set_Uq(U0)
    d = S.rhs_bang(None, g, None, p2de.TimeParam(t, dt, nstage))
    r = g.get_field(abi.FIELD_RHSU)
    g.close()
    return d, r


def _oracle_rhs(desc, U0, t, dt, nstage):
    from oracle.binding import Oracle

    o = Oracle(desc)
    o.set_Uq(U0)
    d = o.rhs(t, dt, nstage)
    r = o.get_field(abi.FIELD_RHSU)
    o.close()
    return d, r


def _noalloc(lib, prm, dmesh, Uq, out, t, dt, nstage, stream):
    out.fill_(float("nan"))
    dto = c_double()
    st = lib.p2de_rhs_noalloc(byref(prm), byref(dmesh), ctypes.c_void_p(Uq.data_ptr()), t, dt, nstage,
                              ctypes.c_void_p(out.data_ptr()), byref(dto), ctypes.c_void_p(stream))
    abi.check(lib, st)
    return dto.value, out.cpu().numpy().copy()


@pytest.mark.parametrize(
    "problem,kw,t,dt",
    [
        (problems.kelvin_helmholtz, dict(N=3, Kx=8, Ky=8, T=0.1), 0.0, 0.05),
        (problems.double_mach_reflection, dict(N=2, Kx=16, Ky=4, T=0.2), 0.01, 1e-4),
        (problems.kelvin_helmholtz, dict(N=3, Kx=8, Ky=8, T=0.1, precision="mixed-acc64"), 0.0, 0.05),
    ],
    ids=["kh-fp64", "dmr-fp64", "kh-mixed-acc64"],
)
def test_rhs_noalloc_matches_regular_entry_point_and_oracle(problem, kw, t, dt):
    import torch

    lib = abi.load_library()
    param, md, bc, desc, U0 = setup(problem, **kw)
    kmax = c_int64()
    abi.check(lib, lib.p2de_noalloc_max_elements(param.N, byref(kmax)))
    assert desc.K <= kmax.value
    arrs = device_mesh_arrays(bc, md.geom)
    dmesh, keep = _device_mesh(torch, arrs, bc)
    Uq = torch.from_numpy(np.ascontiguousarray(U0).ravel()).cuda()
    out = torch.empty_like(Uq)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    calls = []
    free = []
    for nstage in (1, 1, 2):
        calls.append((nstage,) + _noalloc(lib, desc.param, dmesh, Uq, out, t, dt, nstage, stream))
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    # the first call may load the module (and with it the static array); later ones allocate nothing
    assert free[1] == free[0] and free[2] == free[0], free
    for call, (nstage, dto, rhs) in enumerate(calls):
        dref, rref = _regular_rhs(param, md, desc, U0, t, dt, nstage)
        assert abs(dto - dref) <= 1e-13 * abs(dref), (call, dto, dref)
        assert relerr(rhs, rref) <= TOL, (call, relerr(rhs, rref))
        if param.precision == "fp64":
            dora, rora = _oracle_rhs(desc, U0, t, dt, nstage)
            assert abs(dto - dora) <= 1e-13 * abs(dora), (call, dto, dora)
            assert relerr(rhs, rora) <= TOL, (call, relerr(rhs, rora))


def test_rhs_noalloc_rebuilds_the_operator_table_when_zerotol_changes():
    """The operator table in the scratch depends on N and ZEROTOL (entries at or below
    ZEROTOL are dropped); calls that alternate ZEROTOL at the same N each match the regular
    entry point with that ZEROTOL."""
    import torch

    lib = abi.load_library()
    # the intended limiter semantics, under which the high-order volume terms reach rhsU
    # (under the reference's they are limited away and only low-order terms remain)
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=8, Ky=8, T=0.1,
                                    reference_semantics=False, bound=p2de.PositivityBound())
    desc = S.make_descriptor(param, md, bc)
    # a threshold that drops the smallest entries wq D of the N = 3 operator
    param2 = replace(param, global_constants=replace(param.global_constants, ZEROTOL=0.2))
    desc2 = S.make_descriptor(param2, md, bc)
    arrs = device_mesh_arrays(bc, md.geom)
    dmesh, keep = _device_mesh(torch, arrs, bc)
    Uq = torch.from_numpy(np.ascontiguousarray(U0).ravel()).cuda()
    out = torch.empty_like(Uq)
    stream = torch.cuda.current_stream().cuda_stream
    ref = {}
    for p, d in ((param, desc), (param2, desc2)):
        ref[d.param.ZEROTOL] = _regular_rhs(p, md, d, U0, 0.0, 0.05, 2)[1]
    assert relerr(ref[0.2], ref[5e-16]) > 1e-6  # the two thresholds give different operators
    for d in (desc, desc2, desc, desc2):
        _, rhs = _noalloc(lib, d.param, dmesh, Uq, out, 0.0, 0.05, 2, stream)
        assert relerr(rhs, ref[d.param.ZEROTOL]) <= TOL, (d.param.ZEROTOL, relerr(rhs, ref[d.param.ZEROTOL]))


def test_rhs_noalloc_rejects_oversized_and_bad_indices():
    import torch

    lib = abi.load_library()
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=4, Ky=4, T=0.1)
    arrs = device_mesh_arrays(bc, md.geom)
    kmax = c_int64()
    abi.check(lib, lib.p2de_noalloc_max_elements(param.N, byref(kmax)))
    big = abi.P2deParam.from_buffer_copy(desc.param)
    big.K = int(kmax.value) + 1
    dmesh, keep = _device_mesh(torch, arrs, bc)
    Uq = torch.from_numpy(np.ascontiguousarray(U0).ravel()).cuda()
    out = torch.empty_like(Uq)
    dto = c_double()
    st = lib.p2de_rhs_noalloc(byref(big), byref(dmesh), ctypes.c_void_p(Uq.data_ptr()), 0.0, 0.05, 1,
                              ctypes.c_void_p(out.data_ptr()), byref(dto), None)
    assert st == 8  # P2DE_ERR_BUDGET, checked before any launch
    bad = dict(arrs)
    bad["nbr"] = arrs["nbr"].copy()
    bad["nbr"][3] = 10**6
    dmesh2, keep2 = _device_mesh(torch, bad, bc)
    st = lib.p2de_rhs_noalloc(byref(desc.param), byref(dmesh2), ctypes.c_void_p(Uq.data_ptr()), 0.0, 0.05, 1,
                              ctypes.c_void_p(out.data_ptr()), byref(dto), None)
    assert st == 1  # P2DE_ERR_INVALID_ARGUMENT from the index check, before the stage kernels
