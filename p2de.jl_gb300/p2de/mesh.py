"""Uniform quadrilateral meshes with StartUpDG's conventions, as initialize_DG builds
them (src/dg/init.jl:241-252, 265-274) and as make_periodic connects them
(test/test_smoke.jl:22-36).

Arrays mirror Julia's column-major (Nq, K) arrays: a numpy array of shape (K, Nq)
in C order has Julia's memory layout, and so does (K, Nq, 4) for SVector{4} arrays.

Conventions (StartUpDG Quad, SBP/LGL):
  * elements ordered x fastest: k = ex + Kx*ey;
  * nodes i = ir + (N+1)*is (r fastest), r along x, s along y;
  * face nodes: faces r=-1, r=+1, s=-1, s=+1, each ordered along its tangent;
  * mapP holds 1-based linear indices into (Nfp, K); boundary face nodes map to
    themselves until make_periodic connects opposite sides.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np


def gll_rule(N: int) -> tuple[np.ndarray, np.ndarray]:
    """GLL nodes and weights: Newton iteration on (1-x^2)P_N'(x) with the Legendre
    recurrence (Hesthaven & Warburton 2008, sec. 3.2); weights 2/(N(N+1)P_N(x)^2)."""
    Np = N + 1
    x = -np.cos(np.pi * np.arange(Np) / N)

    def legendre(xx):
        P = np.zeros((Np, N + 1))
        P[:, 0] = 1.0
        if N >= 1:
            P[:, 1] = xx
        for k in range(2, N + 1):
            P[:, k] = ((2.0 * k - 1.0) * xx * P[:, k - 1] - (k - 1.0) * P[:, k - 2]) / k
        return P

    for _ in range(100):
        xold = x.copy()
        P = legendre(x)
        x = xold - (x * P[:, N] - P[:, N - 1]) / (Np * P[:, N])
        if np.max(np.abs(x - xold)) < 1e-16:
            break
    for i in range(Np // 2):
        a = 0.5 * (x[Np - 1 - i] - x[i])
        x[i] = -a
        x[Np - 1 - i] = a
    if Np % 2 == 1:
        x[Np // 2] = 0.0
    x[0], x[-1] = -1.0, 1.0
    P = legendre(x)
    w = 2.0 / (N * Np * P[:, N] ** 2)
    return x, w


def gauss_rule(N: int) -> tuple[np.ndarray, np.ndarray]:
    """Gauss-Legendre nodes and weights (gauss_quad(0, 0, N)): Newton iteration on
    P_{N+1} from x_i = -cos(pi (i + 3/4) / (N + 3/2)); weights 2/((1-x^2) P'_{N+1}(x)^2)."""
    n = N + 1

    def legendre(x):
        p0, p1 = np.ones_like(x), x.copy()
        for k in range(2, n + 1):
            p0, p1 = p1, ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k
        dP = n * (x * p1 - p0) / (x * x - 1.0)
        return p1, dP

    x = -np.cos(np.pi * (np.arange(n) + 0.75) / (n + 0.5))
    for _ in range(100):
        P, dP = legendre(x)
        dx = P / dP
        x = x - dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    for i in range(n // 2):
        a = 0.5 * (x[n - 1 - i] - x[i])
        x[i], x[n - 1 - i] = -a, a
    if n % 2 == 1:
        x[n // 2] = 0.0
    _, dP = legendre(x)
    return x, 2.0 / ((1.0 - x * x) * dP * dP)


def face_to_node(N: int) -> np.ndarray:
    """fq2q (0-based): volume node of each face node."""
    n = N + 1
    t = np.arange(n)
    return np.concatenate([n * t, (n - 1) + n * t, t, t + n * (n - 1)])


@dataclass
class MeshData:
    """The fields of StartUpDG's MeshData that P2DE.jl reads, for affine quads."""

    N: int
    K: tuple[int, int]
    xL: tuple[float, float]
    xR: tuple[float, float]
    x: np.ndarray  # (K, Nq) node coordinates
    y: np.ndarray
    xf: np.ndarray  # (K, Nfp) face-node coordinates
    yf: np.ndarray
    mapM: np.ndarray  # (K, Nfp) 1-based
    mapP: np.ndarray  # (K, Nfp) 1-based
    mapB: np.ndarray  # boundary face nodes (1-based), those with mapP == mapM
    geom: np.ndarray  # (K, 5): J, rxJ, sxJ, ryJ, syJ
    sides: dict = field(default_factory=dict)  # 'left','right','bottom','top' -> 1-based face nodes
    dim1: bool = False  # a Line mesh (K = (K, 1), y = 0, two face nodes per element)

    @property
    def xq(self):
        return self.x

    @property
    def yq(self):
        return self.y

    @property
    def num_elements(self) -> int:
        return self.K[0] * self.K[1]

    @property
    def J(self):
        return self.geom[:, 0]


def uniform_mesh(N: int, Kx: int, Ky: int, xL=(0.0, 0.0), xR=(1.0, 1.0), basis: str = "lobatto") -> MeshData:
    """basis "lobatto": nodes and face nodes on the LGL points (RefElemData(Quad(), SBP(), N));
    "gauss": nodes on the Gauss points, face nodes at the face Gauss points (init.jl:83-93)."""
    n = N + 1
    Nq, Nfp = n * n, 4 * n
    K = Kx * Ky
    r, _ = gauss_rule(N) if basis == "gauss" else gll_rule(N)
    hx = (xR[0] - xL[0]) / Kx
    hy = (xR[1] - xL[1]) / Ky
    k = np.arange(K)
    ex, ey = k % Kx, k // Kx
    ir = np.tile(np.arange(n), n)
    is_ = np.repeat(np.arange(n), n)
    x = xL[0] + hx * ex[:, None] + 0.5 * (r[ir][None, :] + 1.0) * hx
    y = xL[1] + hy * ey[:, None] + 0.5 * (r[is_][None, :] + 1.0) * hy
    f = np.arange(Nfp)
    # face f on side f // n (r = -1, r = +1, s = -1, s = +1) at tangential point f % n
    fr = np.where(f // n == 0, -1.0, np.where(f // n == 1, 1.0, r[f % n]))
    fs_ = np.where(f // n == 2, -1.0, np.where(f // n == 3, 1.0, r[f % n]))
    xf = xL[0] + hx * ex[:, None] + 0.5 * (fr[None, :] + 1.0) * hx
    yf = xL[1] + hy * ey[:, None] + 0.5 * (fs_[None, :] + 1.0) * hy
    mapM = 1 + f[None, :] + Nfp * k[:, None]
    side, t = f // n, f % n
    mapP = mapM.copy()
    sides = {}
    # r = -1 face of (ex, ey) <-> r = +1 face of (ex-1, ey), and so on
    for s_, (dx, dy, other) in enumerate([(-1, 0, 1), (1, 0, 0), (0, -1, 3), (0, 1, 2)]):
        fs = f[side == s_]
        nx, ny = ex + dx, ey + dy
        inside = (nx >= 0) & (nx < Kx) & (ny >= 0) & (ny < Ky)
        kn = nx + Kx * ny
        for ff in fs:
            tt = ff % n
            mapP[inside, ff] = 1 + (other * n + tt) + Nfp * kn[inside]
        name = ["left", "right", "bottom", "top"][s_]
        sides[name] = np.sort(np.concatenate([mapM[~inside, ff] for ff in fs]))
    mapB = np.sort(mapM[mapP == mapM])
    geom = np.zeros((K, 5))
    geom[:, 0] = hx * hy / 4.0
    geom[:, 1] = hy / 2.0
    geom[:, 4] = hx / 2.0
    return MeshData(N, (Kx, Ky), tuple(xL), tuple(xR), x, y, xf, yf, mapM, mapP, mapB, geom, sides)


def uniform_mesh_1d(N: int, K: int, xL: float = 0.0, xR: float = 1.0, basis: str = "lobatto",
                    periodic: bool = False) -> MeshData:
    """initialize_uniform_mesh_data(::Line) (init.jl:230-239): K equal elements on [xL, xR],
    nodes on the LGL or Gauss points, face nodes at r = -1, +1; StartUpDG's MeshData for a Line
    maps the two domain ends to themselves unless periodic. geom rows (J, rxJ) = (h/2, 1)."""
    n = N + 1
    r, _ = gauss_rule(N) if basis == "gauss" else gll_rule(N)
    h = (xR - xL) / K
    k = np.arange(K)
    x = xL + h * k[:, None] + 0.5 * (r[None, :] + 1.0) * h
    xf = xL + h * k[:, None] + 0.5 * (np.array([-1.0, 1.0])[None, :] + 1.0) * h
    mapM = 1 + np.arange(2)[None, :] + 2 * k[:, None]
    mapP = mapM.copy()
    mapP[1:, 0] = mapM[:-1, 1]
    mapP[:-1, 1] = mapM[1:, 0]
    if periodic:
        mapP[0, 0], mapP[-1, 1] = mapM[-1, 1], mapM[0, 0]
    mapB = np.sort(mapM[mapP == mapM])
    geom = np.zeros((K, 5))
    geom[:, 0] = h / 2.0
    geom[:, 1] = 1.0
    sides = {"left": np.array([1]) if not periodic else np.array([], dtype=int),
             "right": np.array([2 * K]) if not periodic else np.array([], dtype=int)}
    return MeshData(N, (K, 1), (xL, 0.0), (xR, 0.0), x, np.zeros_like(x), xf, np.zeros_like(xf), mapM, mapP,
                    mapB, geom, sides, dim1=True)


def make_periodic(md: MeshData, periodic=(True, True)) -> MeshData:
    """Connects opposite boundary sides (StartUpDG make_periodic for a uniform mesh)."""
    N = md.N
    n = N + 1
    Nfp = 4 * n
    Kx, Ky = md.K
    K = Kx * Ky
    k = np.arange(K)
    ex, ey = k % Kx, k // Kx
    mapP = md.mapP.copy()
    f = np.arange(Nfp)
    side = f // n
    sides = dict(md.sides)
    if periodic[0]:
        for s_, (dx, other) in enumerate([(-1, 1), (1, 0)]):
            edge = (ex == 0) if dx < 0 else (ex == Kx - 1)
            kn = ((ex + dx) % Kx) + Kx * ey
            for ff in f[side == s_]:
                tt = ff % n
                mapP[edge, ff] = 1 + (other * n + tt) + Nfp * kn[edge]
        sides["left"] = np.zeros(0, dtype=np.int64)
        sides["right"] = np.zeros(0, dtype=np.int64)
    if periodic[1]:
        for s_, (dy, other) in zip((2, 3), [(-1, 3), (1, 2)]):
            edge = (ey == 0) if dy < 0 else (ey == Ky - 1)
            kn = ex + Kx * ((ey + dy) % Ky)
            for ff in f[side == s_]:
                tt = ff % n
                mapP[edge, ff] = 1 + (other * n + tt) + Nfp * kn[edge]
        sides["bottom"] = np.zeros(0, dtype=np.int64)
        sides["top"] = np.zeros(0, dtype=np.int64)
    mapB = np.sort(md.mapM[mapP == md.mapM])
    return replace(md, mapP=mapP, mapB=mapB, sides=sides)


def rotated(md: MeshData, theta: float) -> MeshData:
    """The same elements and connectivity with every node rotated by theta about the
    origin: affine elements whose geometric factors have sxJ, ryJ != 0 (the general,
    not axis-aligned, case of the kernels)."""
    c, s = np.cos(theta), np.sin(theta)
    x, y = c * md.x - s * md.y, s * md.x + c * md.y
    xf, yf = c * md.xf - s * md.yf, s * md.xf + c * md.yf
    g = md.geom.copy()
    rxJ, syJ = md.geom[:, 1], md.geom[:, 4]  # hy/2, hx/2 of the axis-aligned element
    g[:, 1] = c * rxJ      # rxJ =  ys
    g[:, 2] = -s * syJ     # sxJ = -yr
    g[:, 3] = s * rxJ      # ryJ = -xs
    g[:, 4] = c * syJ      # syJ =  xr
    return replace(md, x=x, y=y, xf=xf, yf=yf, geom=g)
