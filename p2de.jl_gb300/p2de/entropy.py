"""The cell entropy inequality of the subcell limiter, evaluated from one stage's fields.

enforce_ES_subcell_volume! (subcell.jl:630-744) lowers interior subcell factors until, for
every element k and direction d,

    sum_{interior subcell faces} L dvdf  <=  rhs_es + max(0, sum_dvfbarL - sum_Bpsi)

with, along each line of the element (initialize_ES_subcell_limiting!, subcell.jl:508-564),
    dvdf         = (v_left - v_right) . (f_bar_H - f_bar_L)   at each interior subcell face,
    sum_dvfbarL  = sum (v_left - v_right) . f_bar_L,
    sum_Bpsi     = sum over the element's face nodes of B_d psi_d(U),
    rhs_es       = sum_Bpsi - sum_dvfbarL, times 1 - beta eps_k for the relaxed bounds (:746-753).
sum_dvfbarL + sum L dvdf is the entropy production estimate of the limited volume fluxes
(entropy_estimate_vol of check_subcell_entropy_stability,
experimental/entropy-stable-limiting.jl:790-955), so the inequality says that the limited
scheme produces no more entropy in the volume than the low-order one or zero, whichever
is larger. This module evaluates both sides with numpy from Uq (the stage's input state),
f_bar_H, f_bar_L and L_local, independently of the kernels that produced them.
"""
from __future__ import annotations

import numpy as np


def v_ufun(U: np.ndarray, gamma: float) -> np.ndarray:
    """Entropy variables (compressible_Navier_Stokes.jl:134-144) of states U[..., 4]."""
    rho, rhou, rhov, E = U[..., 0], U[..., 1], U[..., 2], U[..., 3]
    p = (gamma - 1) * (E - 0.5 * (rhou * rhou + rhov * rhov) / rho)
    s = np.log(p / rho**gamma)
    return np.stack([(gamma + 1 - s) - (gamma - 1) * E / p, rhou * (gamma - 1) / p, rhov * (gamma - 1) / p,
                     -rho * (gamma - 1) / p], axis=-1)


def _face_nodes(n: int):
    """(volume node, side, position along the face) of each face node, faces r=-1, r=+1,
    s=-1, s=+1 in StartUpDG's order."""
    out = []
    for f in range(4 * n):
        side, t = divmod(f, n)
        q = (n * t, (n - 1) + n * t, t, t + n * (n - 1))[side]
        out.append((q, side, t))
    return out


def cell_entropy_sides(Uq, fbarH, fbarL, L_local, geom, N: int, w1D, gamma: float = 1.4, beta_eps=None,
                       relaxed_beta=None):
    """Both sides of the cell entropy inequality per element and direction.

    Uq (K, Nq, 4); fbarH, fbarL (2, K, Nq+N1D, 4) (the layout of P2DE_FIELD_F_BAR_H/L);
    L_local (K, 2, Nq+N1D) (one stage); geom (K, 5) rows (J, rxJ, sxJ, ryJ, syJ); w1D the
    1D quadrature weights of the basis; beta_eps (K,) the relaxed bounds' beta eps_k, or
    None. relaxed_beta: beta of a relaxed bound whose eps_k (in [0, 1]) is not given; the
    target is then the largest over eps_k, max(1, 1 - beta) rhs for rhs >= 0 and
    min(1, 1 - beta) rhs below.
    Returns (lhs, target, scale), each (K, 2): lhs = sum L dvdf, target = rhs_es +
    max(0, sum_dvfbarL - sum_Bpsi), scale = the sum of the magnitudes of every term that
    enters either side (for a rounding tolerance)."""
    n = N + 1
    K = Uq.shape[0]
    U = np.asarray(Uq, dtype=np.float64).reshape(K, n * n, 4)
    fH = np.asarray(fbarH, dtype=np.float64).reshape(2, K, n * (n + 1), 4)
    fL = np.asarray(fbarL, dtype=np.float64).reshape(2, K, n * (n + 1), 4)
    L = np.asarray(L_local, dtype=np.float64).reshape(K, 2, n * (n + 1))
    g = np.asarray(geom, dtype=np.float64).reshape(K, 5)
    v = v_ufun(U, gamma)
    # sum_Bpsi: Bx(dim::Dim2) = (rxJ Br + sxJ Bs, ryJ Br + syJ Bs) with Br = -/+ w on the
    # r = -/+1 faces, Bs likewise on the s faces; psi = (gamma - 1) (rhou, rhov)
    sB = np.zeros((K, 2))
    sBabs = np.zeros((K, 2))
    for q, side, t in _face_nodes(n):
        Br = (-w1D[t], w1D[t], 0.0, 0.0)[side]
        Bs = (0.0, 0.0, -w1D[t], w1D[t])[side]
        for d in range(2):
            Bd = g[:, 1 + 2 * d] * Br + g[:, 2 + 2 * d] * Bs
            term = Bd * ((gamma - 1) * U[:, q, 1 + d])
            sB[:, d] += term
            sBabs[:, d] += np.abs(term)
    lhs = np.zeros((K, 2))
    sdl = np.zeros((K, 2))
    scale = sBabs.copy()
    for d in range(2):
        for a in range(n):
            for b in range(1, n):
                if d == 0:  # x: line sj = a, face si = b between nodes (b-1, a) and (b, a)
                    fi, qm, qp = b + (n + 1) * a, (b - 1) + n * a, b + n * a
                else:  # y: line si = a, face sj = b between nodes (a, b-1) and (a, b)
                    fi, qm, qp = a + n * b, a + n * (b - 1), a + n * b
                dv = v[:, qm, :] - v[:, qp, :]
                dvdf = np.sum(dv * (fH[d, :, fi, :] - fL[d, :, fi, :]), axis=-1)
                lhs[:, d] += L[:, d, fi] * dvdf
                sdl[:, d] += np.sum(dv * fL[d, :, fi, :], axis=-1)
                scale[:, d] += np.sum(np.abs(dv) * (np.abs(fH[d, :, fi, :]) + np.abs(fL[d, :, fi, :])), axis=-1)
    rhs = sB - sdl
    if beta_eps is not None:
        rhs = (1 - np.asarray(beta_eps, dtype=np.float64))[:, None] * rhs
    elif relaxed_beta is not None:
        rhs = np.maximum(rhs, (1 - relaxed_beta) * rhs)
    target = rhs + np.maximum(0.0, sdl - sB)
    return lhs, target, scale


def cell_entropy_violation(*args, zerotol: float = 5e-16, rtol: float = 1e-12, **kw) -> tuple[float, np.ndarray]:
    """The largest (lhs - target - slack) / scale over elements and directions, and the
    (K, 2) mask of those above 0. slack = rtol scale + M zerotol: the greedy repair stops at
    dvdf < ZEROTOL (subcell.jl:676-741), which leaves at most M = N1D (N1D - 1) such terms,
    and both sides are sums that two evaluations round differently."""
    lhs, target, scale = cell_entropy_sides(*args, **kw)
    N = args[5]
    M = (N + 1) * N
    excess = lhs - target - (rtol * scale + M * zerotol)
    worst = float(np.max(excess / np.maximum(scale, 1e-300)))
    return worst, excess > 0
