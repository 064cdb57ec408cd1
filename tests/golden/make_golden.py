"""Generates the regression vectors in tests/golden/ from the FP64 oracle.

The reference ships no golden vectors for this path and Julia is not available to
run it, so these fixtures pin the oracle's own outputs (and, through the GPU tests,
the CUDA path) on small seeded cases: they guard against regressions, they do not
pin parity with P2DE.jl. Run from the repository root:

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "p2de.jl_gb300"))
sys.path.insert(0, str(ROOT))

import p2de  # noqa: E402
from p2de import abi, problems  # noqa: E402
from p2de import solver as S  # noqa: E402
from p2de.types import PositivityBound  # noqa: E402

CASES = {
    "kh_n3_4x4": (problems.kelvin_helmholtz, dict(N=3, Kx=4, Ky=4, T=0.1), 0.0, 0.05),
    "kh_n3_4x4_intended_pos": (
        problems.kelvin_helmholtz,
        dict(N=3, Kx=4, Ky=4, T=0.1, reference_semantics=False, bound=PositivityBound()),
        0.0,
        2e-4,
    ),
    "dmr_n2_8x2": (problems.double_mach_reflection, dict(N=2, Kx=8, Ky=2, T=0.2), 0.0, 1e-3),
    "riemann_n4_3x3": (problems.riemann2d, dict(N=4, Kx=3, Ky=3, T=0.2, seed=5), 0.0, 0.2),
    "vortex_n2_4x4": (problems.isentropic_vortex, dict(N=2, Kx=4, Ky=4), 0.0, 1e-2),
}

FIELDS = {
    "rhsU": abi.FIELD_RHSU,
    "rhsL": abi.FIELD_RHSL,
    "rhsH": abi.FIELD_RHSH,
    "L_local": abi.FIELD_L_LOCAL,
}


def build(name):
    problem, kw, t, dt = CASES[name]
    out = problem(**kw)
    param, ic, bcf = out[0], out[1], out[2]
    md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
    bc = bcf(param, md)
    desc = S.make_descriptor(param, md, bc)
    U0 = S.evaluate_initial_condition(param, md, ic)
    return param, md, bc, desc, U0, t, dt


def compute(name):
    from oracle.binding import Oracle

    param, md, bc, desc, U0, t, dt = build(name)
    o = Oracle(desc, nthreads=1)
    o.set_Uq(U0)
    res = {"U0": U0.ravel().copy(), "t": t, "dt_in": dt}
    res["dt_out"] = o.rhs(t, dt, 1)
    for k, f in FIELDS.items():
        res[k] = o.get_field(f, 1)
    tt, dts = o.step(0.0)
    res["step_dt"] = dts
    res["step_Uq"] = o.get_field(abi.FIELD_UQ)
    o.close()
    return res


def main():
    here = Path(__file__).resolve().parent
    for name in CASES:
        res = compute(name)
        np.savez_compressed(here / f"{name}.npz", **res)
        print(name, {k: np.asarray(v).size for k, v in res.items()})


if __name__ == "__main__":
    main()
