"""Snapshots for ParaView: construct_vtk_file! (src/dg/postprocess.jl:183-216).

Each snapshot of a uniform Kx x Ky mesh is one structured grid of (N+1) Kx by (N+1) Ky
points (the element (ik, jk)'s node (i, j) at point ((ik-1)(N+1) + i, (jk-1)(N+1) + j),
as the reference places them), with point fields rho, rhou, rhov, E; a ParaView
collection (.pvd) lists the snapshots by time. Files are VTK XML, ASCII.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

FIELDS = ("rho", "rhou", "rhov", "E")


def grid_arrays(N: int, K: tuple[int, int], nodal: np.ndarray) -> np.ndarray:
    """(K, Nq, ...) nodal values -> ((N+1) Ky, (N+1) Kx, ...) in the reference's
    placement (elements x-fastest, nodes r-fastest)."""
    n = N + 1
    Kx, Ky = K
    a = np.asarray(nodal).reshape(Ky, Kx, n, n, *np.shape(nodal)[2:])  # [jk][ik][s][r]
    a = np.moveaxis(a, 2, 1)  # [jk][s][ik][r]
    return a.reshape(Ky * n, Kx * n, *np.shape(nodal)[2:])


def _ascii(a: np.ndarray) -> str:
    return " ".join(repr(float(x)) for x in np.ravel(a))


def write_snapshot(path: str | Path, N: int, K: tuple[int, int], x: np.ndarray, y: np.ndarray, Uq: np.ndarray) -> Path:
    """One structured-grid file (.vts) of the state Uq (K, Nq, 4) on nodes x, y (K, Nq). A
    Line state (K, N+1, 3) of CompressibleEulerIdealGas{Dim1} is one row of (N+1) K points
    in element order with fields rho, rhou, E."""
    path = Path(path)
    if path.suffix != ".vts":
        path = path.with_suffix(".vts")
    Uq = np.asarray(Uq)
    fields = FIELDS
    if Uq.size == 3 * np.size(x):  # a Line: nodes in element order along x
        fields = ("rho", "rhou", "E")
        X = np.asarray(x, dtype=np.float64).reshape(1, -1)
        Y = np.zeros_like(X)
        U = Uq.reshape(1, -1, 3)
    else:
        X, Y = grid_arrays(N, K, x), grid_arrays(N, K, y)
        U = grid_arrays(N, K, Uq.reshape(np.shape(x)[0], np.shape(x)[1], 4))
    ny, nx = X.shape
    ext = f"0 {nx - 1} 0 {ny - 1} 0 0"
    pts = np.stack([X, Y, np.zeros_like(X)], axis=-1)
    lines = [
        '<?xml version="1.0"?>',
        '<VTKFile type="StructuredGrid" version="0.1" byte_order="LittleEndian">',
        f'  <StructuredGrid WholeExtent="{ext}">',
        f'    <Piece Extent="{ext}">',
        "      <PointData>",
    ]
    for c, name in enumerate(fields):
        lines.append(f'        <DataArray type="Float64" Name="{name}" format="ascii">{_ascii(U[..., c])}</DataArray>')
    lines += [
        "      </PointData>",
        "      <Points>",
        f'        <DataArray type="Float64" NumberOfComponents="3" format="ascii">{_ascii(pts)}</DataArray>',
        "      </Points>",
        "    </Piece>",
        "  </StructuredGrid>",
        "</VTKFile>",
    ]
    path.write_text("\n".join(lines) + "\n")
    return path


def construct_vtk_file(param, md, data_hist, output_path: str | Path, filename: str) -> Path:
    """construct_vtk_file! (src/dg/postprocess.jl:183-207): one snapshot per entry of
    data_hist (Uhist, thist) and a .pvd collection, named as the reference names them."""
    out = Path(output_path)
    out.mkdir(parents=True, exist_ok=True)
    stem = f"{filename}_N={param.N}_K={tuple(np.atleast_1d(param.K))}"
    entries = []
    for U, t in zip(data_hist.Uhist, data_hist.thist):
        f = write_snapshot(out / f"{stem}_t={t}.vts", param.N, param.K, md.x, md.y, U)
        entries.append((t, f.name))
    pvd = out / f"{stem}.pvd"
    body = "\n".join(f'    <DataSet timestep="{t!r}" part="0" file="{name}"/>' for t, name in entries)
    pvd.write_text(
        '<?xml version="1.0"?>\n<VTKFile type="Collection" version="0.1" byte_order="LittleEndian">\n'
        f"  <Collection>\n{body}\n  </Collection>\n</VTKFile>\n"
    )
    return pvd


def read_snapshot(path: str | Path) -> dict:
    """The point fields and coordinates of a file written by write_snapshot."""
    import xml.etree.ElementTree as ET

    root = ET.parse(str(path)).getroot()
    piece = root.find("StructuredGrid/Piece")
    e = [int(v) for v in piece.get("Extent").split()]
    shape = (e[3] - e[2] + 1, e[1] - e[0] + 1)
    out = {}
    for da in piece.find("PointData"):
        out[da.get("Name")] = np.array(da.text.split(), dtype=np.float64).reshape(shape)
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=np.float64).reshape(*shape, 3)
    out["x"], out["y"] = pts[..., 0], pts[..., 1]
    return out
