"""The C ABI library loads and exports every entry point include/p2de.h declares;
host-side argument checks answer with status codes (CPU only, no compute calls)."""
import ctypes
import re
from ctypes import byref, c_int64, c_void_p
from pathlib import Path

import numpy as np
import pytest

import p2de
from p2de import abi, problems
from p2de import solver as S

from conftest import has_gpu
from helpers import setup

HEADER = Path(__file__).resolve().parents[1] / "include" / "p2de.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(p2de_\w+)\s*\(", text)))


def test_header_declares_the_binding_list():
    names = declared_functions()
    assert names == sorted(n for n, _, _ in abi.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(abi.LIB_PATH))
    for name in declared_functions():
        assert hasattr(lib, name), name
    lib2 = abi.load_library()
    assert lib2.p2de_abi_version() == 5


def test_field_counts():
    lib = abi.load_library()
    c = c_int64()
    assert lib.p2de_field_count(3, 10, abi.FIELD_UQ, byref(c)) == 0 and c.value == 4 * 16 * 10
    assert lib.p2de_field_count(3, 10, abi.FIELD_BF_H, byref(c)) == 0 and c.value == 8 * 16 * 10
    assert lib.p2de_field_count(3, 10, abi.FIELD_L_LOCAL, byref(c)) == 0 and c.value == 20 * 2 * 10
    assert lib.p2de_field_count(3, 10, abi.FIELD_L, byref(c)) == 0 and c.value == 10
    assert lib.p2de_field_count(6, 10, abi.FIELD_UQ, byref(c)) == 1  # N outside 1..5
    assert lib.p2de_field_count(3, 10, 42, byref(c)) == 1


def test_invalid_arguments_are_rejected_before_the_device():
    lib = abi.load_library()
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=3, Ky=3, T=0.1)
    h = c_void_p()
    # mapP out of range
    bad = desc.keep[1].copy()
    bad[5] = 10**9
    m = abi.P2deMesh.from_buffer_copy(desc.mesh)
    m.mapP = abi.iptr(bad)
    st = lib.p2de_initialize_DG(byref(desc.param), byref(m), 0, byref(h))
    assert st == 1 and "mapP" in abi.last_error(lib, None)
    # unsupported degree
    p = abi.P2deParam.from_buffer_copy(desc.param)
    p.N = 6
    assert lib.p2de_initialize_DG(byref(p), byref(desc.mesh), 0, byref(h)) == 1
    # non-positive Jacobian
    geom = desc.keep[0].copy()
    geom[2, 0] = 0.0
    m2 = abi.P2deMesh.from_buffer_copy(desc.mesh)
    m2.geom = abi.dptr(geom)
    assert lib.p2de_initialize_DG(byref(desc.param), byref(m2), 0, byref(h)) == 1
    # null pointers
    assert lib.p2de_initialize_DG(None, byref(desc.mesh), 0, byref(h)) == 1
    assert lib.p2de_rhs(None, 0.0, 0.0, 1, None) == 1


@pytest.mark.skipif(has_gpu(), reason="checks the no-device answer")
def test_no_device_is_a_status_not_a_crash():
    lib = abi.load_library()
    param, md, bc, desc, U0 = setup(problems.kelvin_helmholtz, N=3, Kx=3, Ky=3, T=0.1)
    h = c_void_p()
    st = lib.p2de_initialize_DG(byref(desc.param), byref(desc.mesh), 0, byref(h))
    assert st == 7  # P2DE_ERR_NO_DEVICE
    with pytest.raises(p2de.P2deError):
        S.Solver(param, md, desc)


def test_line_descriptors_checked_before_the_device():
    """CompressibleEulerIdealGas{Dim1} descriptors are checked on the host: what the Line
    path refuses comes back as P2DE_ERR_UNSUPPORTED (2) or INVALID_ARGUMENT (1) with no
    device; an accepted one reaches the device query (P2DE_ERR_NO_DEVICE, 7, here)."""
    from ctypes import byref, c_void_p

    from p2de import problems
    from p2de.types import GaussCollocation, NodewiseScaledExtrapolation, PositivityAndCellEntropyBound, SubcellLimiter

    from helpers import setup

    lib = abi.load_library()

    def status(desc):
        h = c_void_p()
        return lib.p2de_initialize_DG(byref(desc.param), byref(desc.mesh), 0, byref(h))

    ok = setup(problems.leblanc, N=2, K=8)[3]
    assert status(ok) in (0, 7)
    refsem = setup(problems.leblanc, N=2, K=8)[3]
    refsem.param.reference_semantics = 1
    assert status(refsem) == 2
    gauss_cell = setup(problems.leblanc, N=2, K=8, approximation_basis=GaussCollocation(),
                       entropyproj_limiter=NodewiseScaledExtrapolation(),
                       rhs_limiter=SubcellLimiter(bound=PositivityAndCellEntropyBound()))[3]
    assert status(gauss_cell) == 2
    mixed = setup(problems.leblanc, N=2, K=8)[3]
    mixed.param.precision = 1
    assert status(mixed) == 2
    bad_map = setup(problems.leblanc, N=2, K=8)
    desc = bad_map[3]
    desc.keep[1][3] = 99  # a mapP entry outside 1..2K
    assert status(desc) == 1
