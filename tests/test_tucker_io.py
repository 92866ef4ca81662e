"""Tucker density files in the reference's format (main.cc:1528-1632 writes,
dft/InitialGuess.cc:764-904 and 1211-1307 read): round trips, the clamped
cubic spline of the reader, the written ranks and a density evaluated at the
quadrature points of the FEM grid."""
import numpy as np
import pytest

from ttdft_public_gb300 import system, tucker_io


def test_core_and_factor_files_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    core = rng.standard_normal((3, 4, 5))
    coords = np.linspace(-2.0, 3.0, 7)
    U = rng.standard_normal((7, 3))
    tucker_io.write_core(str(tmp_path / "c"), core)
    tucker_io.write_factor(str(tmp_path / "f"), coords, U)
    assert np.array_equal(tucker_io.read_core(str(tmp_path / "c")), core)
    x, V = tucker_io.read_factor(str(tmp_path / "f"))
    assert np.array_equal(x, coords) and np.array_equal(V, U)
    # the core file lists x fastest
    with open(tmp_path / "c") as f:
        lines = f.read().split("\n")
    assert lines[0] == "3 4 5"
    assert float(lines[1 + 1]) == core[1, 0, 0] and float(lines[1 + 3]) == core[0, 1, 0]


def test_truncated_files_are_rejected(tmp_path):
    p = tmp_path / "c"
    p.write_text("2 2 2\n1.0\n2.0\n")
    with pytest.raises(ValueError):
        tucker_io.read_core(str(p))


def test_clamped_spline_interpolates_with_flat_ends():
    x = np.array([0.0, 0.3, 0.45, 0.7, 1.0])
    y = np.sin(3 * x) + x ** 2
    s = tucker_io.ClampedCubic(x, y)
    assert np.allclose(s(x)[:, 0], y, atol=1e-14)
    eps = 1e-7    # one-sided difference: error ~ s'' eps / 2
    for x0, sign in ((0.0, 1), (1.0, -1)):
        d = (s(np.array([x0 + sign * eps]))[0, 0] - s(np.array([x0]))[0, 0]) / (sign * eps)
        assert abs(d) < 1e-5
    # a cubic with zero end slopes is reproduced exactly
    p = lambda t: 2 * t ** 3 - 3 * t ** 2
    t = np.linspace(0, 1, 101)
    assert np.allclose(tucker_io.ClampedCubic(x, p(x))(t)[:, 0], p(t), atol=1e-13)


def test_clamped_spline_matches_scipy():
    interpolate = pytest.importorskip("scipy.interpolate")
    rng = np.random.default_rng(2)
    x = np.sort(rng.uniform(0, 10, 12))
    y = rng.standard_normal((12, 3))
    t = np.linspace(x[0], x[-1], 200)
    ref = interpolate.CubicSpline(x, y, bc_type="clamped")(t)    # zero end slopes
    assert np.abs(tucker_io.ClampedCubic(x, y)(t) - ref).max() < 1e-12 * np.abs(ref).max()


def test_output_ranks_rule():
    # int(100 log n / log 250), or int(0.6 n) when not below n (main.cc:1543-1557)
    assert tucker_io.output_ranks([241, 121, 61]) == [99, 86, 36]


def test_density_from_files_at_quadrature_points(tmp_path):
    """A separable density with flat ends, written at the FEM nodes and read
    back, evaluated at the quadrature points as the reference's initial guess
    does: spline accuracy on the node spacing."""
    fem = [system.Fem1D(20, -5.0, 5.0) for _ in range(3)]
    g = lambda t: np.cos(np.pi * t / 10.0) ** 2 + 0.1        # g'(+-5) = 0
    U = [g(f.nodes)[:, None] for f in fem]
    core = np.full((1, 1, 1), 2.0)
    names = tucker_io.write_density(str(tmp_path), core, [f.nodes for f in fem], U, [8, 8, 8])
    assert [n.split("/")[-1] for n in names] == ["rank_8_core", "rank_8_factor_x",
                                                "rank_8_factor_y", "rank_8_factor_z"]
    for src, dst in zip(names, [tucker_io.CORE_IN, *tucker_io.FACTOR_IN]):
        (tmp_path / dst).write_text(open(src).read())
    c, fac = tucker_io.read_density(str(tmp_path))
    Uq = [tucker_io.factors_at(x, u, f.xq) for (x, u), f in zip(fac, fem)]
    rho = tucker_io.reconstruct(c, Uq)
    exact = 2.0 * np.einsum("i,j,k->ijk", *[g(f.xq) for f in fem])
    assert np.abs(rho - exact).max() < 1e-4 * exact.max()
