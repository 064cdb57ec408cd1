"""The seeded workload generators of the batched and served runs: reproducible, and
drawn from the stated ranges; the error and entropy helpers on known inputs."""
import numpy as np

from p2de import workloads as W


def test_riemann_batch_is_seeded_and_in_range():
    a, b = W.riemann_batch_cases(64, seed=3), W.riemann_batch_cases(64, seed=3)
    assert a == b and len(a) == 64
    assert {c.K1d for c in a} <= {32, 64, 128, 192}
    assert {c.N for c in a} <= {2, 3, 4}
    assert all(0.1 <= c.T <= 0.3 and c.family == "riemann" for c in a)
    assert len({c.seed for c in a}) == 64
    assert W.riemann_batch_cases(64, seed=4) != a


def test_serving_stream_is_poisson_and_in_range():
    s = W.serving_stream(2000, 50.0, seed=5)
    arr = np.array([c.arrival for c in s])
    assert np.all(np.diff(arr) > 0)
    gaps = np.diff(np.concatenate([[0.0], arr]))
    assert abs(gaps.mean() - 1 / 50.0) < 0.1 / 50.0  # mean inter-arrival 1/rate
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.1  # exponential: cv = 1
    assert {c.family for c in s} == {"kh", "riemann", "vortex"}
    assert {c.N for c in s} == {2, 3, 4, 5}
    assert {c.K1d for c in s} == set(W.SERVING_MESHES)
    assert all(0.05 <= c.T <= 0.5 for c in s)
    for c in s:
        if c.family == "vortex":
            assert 1 <= c.extra["strength"] <= 5 and 0 <= c.extra["ux"] <= 1 and 0 <= c.extra["uy"] <= 1
    half = W.serving_stream(50, 50.0, seed=5, time_scale=0.5)
    assert all(abs(h.T - 0.5 * f.T) < 1e-15 for h, f in zip(half, s[:50]))


def test_build_case_shapes_and_states():
    for c in [W.Case("riemann", 2, 8, 0.1, 7), W.Case("kh", 3, 4, 0.1, 1),
              W.Case("vortex", 4, 4, 0.1, 0, extra={"strength": 3.0, "ux": 0.5, "uy": 0.2})]:
        param, md, bc, desc, U0 = W.build_case(c, "mixed")
        assert U0.shape == (c.K1d**2, (c.N + 1) ** 2, 4)
        assert desc.param.precision == 1
        assert np.all(U0[..., 0] > 0)


def test_errors_and_entropy_helpers():
    c = W.Case("kh", 2, 4, 0.1, 1)
    param, md, bc, desc, U0 = W.build_case(c)
    Wq = W.quadrature_weights(2, md.geom)
    assert abs(Wq.sum() - 1.0) < 1e-13  # area of [0,1]^2
    e = W.relative_errors(U0, U0, Wq)
    assert all(v["L1"] == 0 and v["Linf"] == 0 for v in e.values())
    U1 = U0.copy()
    U1[..., 0] *= 1 + 1e-6
    assert abs(W.relative_errors(U1, U0, Wq)["rho"]["L1"] - 1e-6) < 1e-12
    # entropy of a uniform state: -rho s/(gamma-1) times the area
    U = np.zeros_like(U0)
    U[..., 0], U[..., 3] = 2.0, 2.5 / 0.4
    s = np.log(2.5) - 1.4 * np.log(2.0)
    assert abs(W.total_entropy(U, Wq) - (-2.0 * s / 0.4)) < 1e-12
