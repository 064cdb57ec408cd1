"""Snapshot writer (construct_vtk_file!, src/dg/postprocess.jl:183-216): the reference's
point placement and a write/read round trip; no GPU."""
import numpy as np

import p2de
from p2de import postprocess as P
from p2de.types import DataHistory


def test_grid_placement_follows_the_reference():
    N, Kx, Ky = 2, 3, 2
    md = p2de.uniform_mesh(N, Kx, Ky, (0.0, 0.0), (3.0, 2.0))
    X, Y = P.grid_arrays(N, (Kx, Ky), md.x), P.grid_arrays(N, (Kx, Ky), md.y)
    n = N + 1
    assert X.shape == (Ky * n, Kx * n)
    assert np.all(np.diff(X, axis=1) >= 0) and np.all(np.diff(Y, axis=0) >= 0)
    assert np.all(np.diff(X, axis=0) == 0) and np.all(np.diff(Y, axis=1) == 0)
    # element k = ik + Kx jk, node i = r + n s  ->  point (jk n + s, ik n + r)
    for k in range(Kx * Ky):
        ik, jk = k % Kx, k // Kx
        for m in range((N + 1) ** 2):
            r, s = m % n, m // n
            assert X[jk * n + s, ik * n + r] == md.x[k, m]
            assert Y[jk * n + s, ik * n + r] == md.y[k, m]


def test_snapshot_round_trip(tmp_path):
    N, Kx, Ky = 3, 4, 3
    md = p2de.uniform_mesh(N, Kx, Ky)
    rng = np.random.default_rng(1)
    U = rng.uniform(0.5, 2.0, size=(Kx * Ky, (N + 1) ** 2, 4))
    f = P.write_snapshot(tmp_path / "snap", N, (Kx, Ky), md.x, md.y, U)
    back = P.read_snapshot(f)
    G = P.grid_arrays(N, (Kx, Ky), U)
    for c, name in enumerate(P.FIELDS):
        np.testing.assert_array_equal(back[name], G[..., c])
    np.testing.assert_array_equal(back["x"], P.grid_arrays(N, (Kx, Ky), md.x))


def test_collection_lists_every_snapshot(tmp_path):
    param, ic, bcf = p2de.problems.kelvin_helmholtz(N=1, Kx=2, Ky=2, T=0.1)
    md = p2de.uniform_mesh(param.N, *param.K, param.xL, param.xR)
    U = np.ones((4, 4, 4))
    hist = DataHistory(Uhist=[U, 2 * U], Lhist=[], thetahist=[], thist=[0.0, 0.1], dthist=[])
    pvd = P.construct_vtk_file(param, md, hist, tmp_path, "kh")
    text = pvd.read_text()
    assert text.count("<DataSet") == 2 and 'timestep="0.1"' in text
    files = sorted(p.name for p in tmp_path.glob("*.vts"))
    assert len(files) == 2
    np.testing.assert_array_equal(P.read_snapshot(tmp_path / files[1])["rho"], 2.0)


def test_line_snapshot_round_trip(tmp_path):
    """A Line state (K, N+1, 3) is written as one row of points in element order."""
    from p2de import problems
    from p2de.mesh import uniform_mesh_1d

    md = uniform_mesh_1d(3, 5, -1.0, 1.0)
    eq = problems.line_param(3, 5, -1.0, 1.0, 0.1).equation
    U = problems.primitive_to_conservative(eq, problems.density_wave_1d_exact(None, md.x, 0.0))
    f = P.write_snapshot(tmp_path / "line", 3, (5, 1), md.x, md.y, U)
    back = P.read_snapshot(f)
    assert set(back) == {"rho", "rhou", "E", "x", "y"}
    np.testing.assert_array_equal(back["x"].ravel(), md.x.ravel())
    np.testing.assert_array_equal(back["rho"].ravel(), U[..., 0].ravel())
    np.testing.assert_array_equal(back["E"].ravel(), U[..., 2].ravel())
