"""Seeded workloads of many independent solves.

riemann_batch_cases: independent four-quadrant Riemann problems on [0,1]^2 with outflow
  boundaries; quadrant states rho ~ U[0.1, 2], p ~ U[0.02, 2], u, v ~ U[-1, 1]; meshes of
  32^2, 64^2, 128^2 or 192^2 quads; N in {2, 3, 4}; t_final ~ U[0.1, 0.3].
serving_stream: a Poisson arrival stream of solves from three families (Kelvin-Helmholtz,
  four-quadrant Riemann, isentropic vortex of strength U[1, 5] advected at U[0, 1]^2),
  meshes of 16^2 .. 256^2 quads, N in 2..5, t_final ~ U[0.05, 0.5] (times an optional
  time scale).

Every draw comes from numpy's PCG64 with the given seed, so the same seed gives the same
cases on every machine.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import problems
from .mesh import gll_rule, uniform_mesh
from . import solver as S


@dataclass
class Case:
    family: str  # "riemann", "kh" or "vortex"
    N: int
    K1d: int  # K1d x K1d quads
    T: float
    seed: int
    arrival: float = 0.0  # seconds after the stream starts
    extra: dict = field(default_factory=dict)

    @property
    def nodes(self) -> int:
        return self.K1d * self.K1d * (self.N + 1) ** 2


def riemann_batch_cases(n: int = 64, seed: int = 3) -> list[Case]:
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        K1d = int(rng.choice([32, 64, 128, 192]))
        N = int(rng.choice([2, 3, 4]))
        T = float(rng.uniform(0.1, 0.3))
        out.append(Case("riemann", N, K1d, T, int(rng.integers(0, 2**31 - 1))))
    return out


SERVING_MESHES = (16, 32, 64, 128, 256)


def serving_stream(n: int, rate: float, seed: int = 5, time_scale: float = 1.0, meshes=SERVING_MESHES) -> list[Case]:
    """n requests with exponential inter-arrival times of mean 1/rate seconds."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for _ in range(n):
        t += float(rng.exponential(1.0 / rate))
        fam = ("kh", "riemann", "vortex")[int(rng.integers(0, 3))]
        K1d = int(rng.choice(meshes))
        N = int(rng.integers(2, 6))
        T = float(rng.uniform(0.05, 0.5)) * time_scale
        s = int(rng.integers(0, 2**31 - 1))
        extra = {}
        if fam == "vortex":
            extra = {"strength": float(rng.uniform(1.0, 5.0)), "ux": float(rng.uniform(0.0, 1.0)),
                     "uy": float(rng.uniform(0.0, 1.0))}
        out.append(Case(fam, N, K1d, T, s, arrival=t, extra=extra))
    return out


def build_case(case: Case, precision: str = "fp64"):
    """(param, md, bc, desc, U0) of a case."""
    kw = dict(N=case.N, Kx=case.K1d, Ky=case.K1d, T=case.T, precision=precision)
    if case.family == "riemann":
        param, ic, bcf = problems.riemann2d(seed=case.seed, **kw)
    elif case.family == "kh":
        param, ic, bcf = problems.kelvin_helmholtz(seed=case.seed, **kw)
    elif case.family == "vortex":
        param, ic, bcf, _ = problems.isentropic_vortex(**case.extra, **kw)
    else:
        raise ValueError(f"unknown family {case.family}")
    md = S.mesh_for(param)
    bc = bcf(param, md)
    desc = S.make_descriptor(param, md, bc)
    U0 = S.evaluate_initial_condition(param, md, ic)
    return param, md, bc, desc, U0


def quadrature_weights(N: int, geom: np.ndarray) -> np.ndarray:
    """(K, Nq) weights J * wq of the tensor-product LGL rule (node i = a + N1D b)."""
    _, w = gll_rule(N)
    n = N + 1
    wq = w[np.tile(np.arange(n), n)] * w[np.repeat(np.arange(n), n)]
    return geom[:, 0:1] * wq[None, :]


def total_entropy(U: np.ndarray, W: np.ndarray, gamma: float = 1.4) -> float:
    """Integral of the entropy -rho s / (gamma - 1), s = log(p / rho^gamma)."""
    U = U.reshape(W.shape[0], W.shape[1], 4)
    rho = U[..., 0]
    p = (gamma - 1) * (U[..., 3] - 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2) / rho)
    s = np.log(p) - gamma * np.log(rho)
    return float(np.sum(W * (-rho * s / (gamma - 1))))


def relative_errors(U: np.ndarray, Uref: np.ndarray, W: np.ndarray) -> dict:
    """Relative L1 (quadrature-weighted) and Linf errors per component."""
    U = U.reshape(W.shape[0], W.shape[1], 4)
    R = Uref.reshape(W.shape[0], W.shape[1], 4)
    out = {}
    for c, name in enumerate(("rho", "rhou", "rhov", "E")):
        d = np.abs(U[..., c] - R[..., c])
        l1r = float(np.sum(W * np.abs(R[..., c])))
        out[name] = {
            "L1": float(np.sum(W * d)) / (l1r if l1r > 0 else 1.0),
            "Linf": float(d.max()) / max(float(np.abs(R[..., c]).max()), 1e-300),
        }
    return out
