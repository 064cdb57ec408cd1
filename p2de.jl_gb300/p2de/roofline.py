"""Algorithmic work of the stage kernels, for the roofline figures.

Stage kernel A is bound by the FP64 pipe (GB300 runs FP64 at 1/58 of its FP32 rate),
so its roofline is in FP64 TFLOP/s. The work below counts one operation per IEEE
operation written in the kernel source (+, -, *, /, sqrt, log, fabs, min/max,
compare), an FMA-contractible a*b+c as two; a division, square root or logarithm
counts as ONE operation although the FP64 pipe spends several instructions on it,
so the fraction of peak understates how busy the pipe is. The data-dependent part
(the quadratic internal-energy solves that the exact l == 0 shortcut skips) is
counted from the kernel's own counter of solves evaluated.

Per element and stage, with n = N+1, Nq = n^2, Nfp = 4n, low-order pairs
NPL = 2n(n-1), high-order pairs NPH = n^2(n-1), subcell faces NSF = n(n+1):
  nodes: primitives, fluxes, two wavespeeds, two logs          50 Nq
  low-order pairs: lambda, averaged flux, viscosity             31 NPL
  gather of the low-order pairs (8 adds + lambda per side)       8 Nq + 18 NPL
  surface (neighbour wavespeed, fluxes, LF, B f*)               74 Nfp
  low-order finish (face terms, 1/(wq J), CFL)                  17 Nq + 9 Nfp
  high-order pairs: Chandrashekar flux with two log-means       52 NPH
  gather and lift of the high-order pairs                       24 Nq + 16 NPH + 16 Nfp
  subcell prefix sums and the low-order update                  55 Nq
  bound evaluations (P[0], density bound)                       10 * 4 Nq
  quadratic solves evaluated (P vector, a, b, c, roots)         51 each
  combine per face                                               4 NSF
"""
from __future__ import annotations


def stage_a_flops_per_elem(N: int) -> int:
    n = N + 1
    Nq, Nfp = n * n, 4 * n
    NPL, NPH, NSF = 2 * n * (n - 1), n * n * (n - 1), n * (n + 1)
    return (
        50 * Nq
        + 31 * NPL
        + 8 * Nq + 18 * NPL
        + 74 * Nfp
        + 17 * Nq + 9 * Nfp
        + 52 * NPH
        + 24 * Nq + 16 * NPH + 16 * Nfp
        + 55 * Nq
        + 10 * 4 * Nq
        + 4 * NSF
    )


FLOPS_PER_QUAD_SOLVE = 51


def stage_a_flops(N: int, K: int, quad_solves: float) -> float:
    """FP64 operations of one launch of stage kernel A over K elements."""
    return stage_a_flops_per_elem(N) * K + FLOPS_PER_QUAD_SOLVE * quad_solves


def stage_bytes(N: int, K: int) -> dict:
    """Compulsory HBM bytes per launch (each input read once, each output written once)."""
    n = N + 1
    Nq, Nfp, NSF = n * n, 4 * n, n * (n + 1)
    a = K * (32 * Nq + 32 * Nfp + 40 + 8 * 16 * NSF + 8 * 2 * NSF)
    b = K * (8 * 2 * NSF + 8 * 4 * n + 8 * 16 * NSF + 3 * 32 * Nq + 2 * 32 * Nq + 8 * 2 * NSF + 8)
    return {"stage_a": a, "stage_b": b}
