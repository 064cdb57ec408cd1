"""p2de_rhs_noalloc: the right-hand side for callers that cannot allocate device memory
(a process whose HBM is reserved by its own pool, or code running during CUDA-graph
capture, where cudaMalloc is not allowed). The test owns every device buffer (allocated
here with torch); the entry point runs with only its static scratch array. Its output
must equal the regular entry point's (p2de_rhs on a solver handle) within the parity
tolerance, on two calls in a row, which also checks that the shared scratch carries
nothing over from one call to the next. This file is collected last so that a run that
stops at its first failure has already run every other test."""
import ctypes
from ctypes import byref, c_double, c_int64

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


@pytest.mark.parametrize(
    "problem,kw,t,dt",
    [
        (problems.kelvin_helmholtz, dict(N=3, Kx=8, Ky=8, T=0.1), 0.0, 0.05),
        (problems.double_mach_reflection, dict(N=2, Kx=16, Ky=4, T=0.2), 0.01, 1e-4),
    ],
)
def test_rhs_noalloc_matches_regular_entry_point_twice(problem, kw, t, dt):
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
    for call, nstage in enumerate((1, 1, 2)):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        dto = c_double()
        st = lib.p2de_rhs_noalloc(
            byref(desc.param), byref(dmesh), ctypes.c_void_p(Uq.data_ptr()), t, dt, nstage,
            ctypes.c_void_p(out.data_ptr()), byref(dto), ctypes.c_void_p(stream),
        )
        abi.check(lib, st)
        dref, rref = _regular_rhs(param, md, desc, U0, t, dt, nstage)
        assert abs(dto.value - dref) <= 1e-13 * abs(dref), (call, dto.value, dref)
        e = relerr(out.cpu().numpy(), rref)
        assert e <= TOL, (call, e)


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
