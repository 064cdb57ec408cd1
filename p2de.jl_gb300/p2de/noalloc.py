"""Host-side helpers for p2de_rhs_noalloc: the device-mesh arrays (exterior indices,
boundary codes) that p2de_initialize_DG builds internally, as numpy arrays the caller
uploads into memory it already owns."""
from __future__ import annotations

import numpy as np

from .types import BCData

BC_INTERIOR, BC_INFLOW, BC_OUTFLOW, BC_WALL, BC_SHOCK = 0, 1, 2, 3, 4


def device_mesh_arrays(bc: BCData, geom: np.ndarray) -> dict:
    """nbr (int32, mapP - 1), bc codes (int8), bcidx (int32), Ival, xyS, geom and the
    axis_aligned flag, in the layouts of p2de_device_mesh."""
    mapP = np.asarray(bc.mapP, dtype=np.int64).ravel()
    nfk = mapP.size
    code = np.zeros(nfk, dtype=np.int8)
    idx = np.zeros(nfk, dtype=np.int32)
    mapI = np.asarray(bc.mapI, dtype=np.int64).ravel()
    code[mapI - 1] = BC_INFLOW
    idx[mapI - 1] = np.arange(mapI.size, dtype=np.int32)
    code[np.asarray(bc.mapO, dtype=np.int64).ravel() - 1] = BC_OUTFLOW
    code[np.asarray(bc.mapW, dtype=np.int64).ravel() - 1] = BC_WALL
    mapS = np.asarray(bc.mapS, dtype=np.int64).ravel()
    code[mapS - 1] = BC_SHOCK
    idx[mapS - 1] = np.arange(mapS.size, dtype=np.int32)
    g = np.ascontiguousarray(geom, dtype=np.float64)
    Ival = np.ascontiguousarray(np.asarray(bc.Ival if len(bc.Ival) else np.zeros((1, 4)), dtype=np.float64).reshape(-1, 4))
    xyS = np.ascontiguousarray(np.asarray(bc.xyS if len(bc.xyS) else np.zeros((1, 2)), dtype=np.float64).reshape(-1, 2))
    return {
        "geom": g,
        "nbr": (mapP - 1).astype(np.int32),
        "bc": code,
        "bcidx": idx,
        "Ival": Ival,
        "nI": mapI.size,
        "xyS": xyS,
        "nS": mapS.size,
        "axis_aligned": int(np.all(g[:, 2] == 0.0) and np.all(g[:, 3] == 0.0)),
    }
