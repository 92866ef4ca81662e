"""The Poisson/FEM Hartree fallback of the oracle (oracle/poisson.py): the
extended mesh, and the potential of known charges against closed forms and
against the kernel-expansion Hartree potential."""
import numpy as np
import scipy.special

import oracle
from oracle import poisson
from ttdft_public_gb300 import system
from ttdft_public_gb300.kernel_expansion import coulomb_expansion


def test_extended_mesh_grows_geometrically():
    e = poisson.extended_edges(0.0, 10.0, 16, 8, 1.5, -40.0, 50.0)
    assert e.size == 16 + 8 + 1
    assert np.isclose(e[0], -40.0) and np.isclose(e[-1], 50.0)
    assert np.allclose(e[4:21], np.linspace(0, 10, 17))
    right = np.diff(e[20:])
    assert np.allclose(right[1:] / right[:-1], 1.5)
    assert np.allclose(np.diff(e[:5])[::-1], right)


def _gaussian_case(n_el, Q=3.0, w=1.0, c=(5.0, 5.0, 5.0)):
    fem = system.Fem1D(n_el, 0.0, 10.0)
    Z, Y, X = np.meshgrid(fem.xq, fem.xq, fem.xq, indexing="ij")
    r = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2)
    rho = Q / (np.pi * w * w) ** 1.5 * np.exp(-r ** 2 / w ** 2)
    return fem, rho, Q * scipy.special.erf(r / w) / r


def test_gaussian_charge_against_closed_form():
    """A Gaussian charge's potential Q erf(r/w)/r; the error falls with the
    mesh (measured 2.3e-3 -> 4.3e-4 of the maximum from 16 to 32 elements,
    relative L2 5.5e-4 at 16)."""
    errs = []
    for n_el in (16, 32):
        fem, rho, exact = _gaussian_case(n_el)
        edges = [np.linspace(0, 10, n_el + 1)] * 3
        phi, info = poisson.solve_hartree(rho, edges, [[3.0, 5.0, 5.0, 5.0]], n_outer=12,
                                          coarsening=1.4)
        assert info["residual"] <= 1e-10
        errs.append(np.abs(phi - exact).max() / np.abs(exact).max())
        if n_el == 16:
            assert np.linalg.norm(phi - exact) / np.linalg.norm(exact) < 1e-3
    assert errs[0] < 3e-3 and errs[1] < errs[0] / 3


def test_two_atom_superposition_density_against_closed_form():
    """The superposition density of the 2-atom test system is a sum of
    Gaussian atoms, whose potential is sum_a Z erf(r_a / w) / r_a (measured
    4.7e-4 relative L2)."""
    spec = system.small_spec(n_el=16, rank=8)
    s = system.build_system(spec)
    grids = [b.fem.xq for b in s.basis]
    rho = oracle.sad_density(s.atoms, grids, spec.z_val, 1.0)
    edges = [np.linspace(b.fem.x0, b.fem.x1, b.fem.n_el + 1) for b in s.basis]
    nuclei = [[spec.z_val, *a] for a in s.atoms]
    phi, info = poisson.solve_hartree(rho, edges, nuclei, n_outer=12, coarsening=1.4)
    Z, Y, X = np.meshgrid(grids[2], grids[1], grids[0], indexing="ij")
    exact = np.zeros_like(rho)
    for a in s.atoms:
        r = np.sqrt((X - a[0]) ** 2 + (Y - a[1]) ** 2 + (Z - a[2]) ** 2)
        exact += spec.z_val * scipy.special.erf(r) / r
    assert np.linalg.norm(phi - exact) / np.linalg.norm(exact) < 2e-3


def test_kernel_expansion_converges_to_the_poisson_potential():
    """The cross-check the fallback exists for: the kernel-expansion Hartree
    potential (the default path, KSDFTPotential.cc:269-340) integrates its
    narrow Gaussian terms by the quadrature rule, so it converges to the
    potential with the quadrature.  A unit-width Gaussian charge, 3-point
    Gauss: relative L2 error 0.17 with 0.625-bohr elements, 0.013 with
    0.27-bohr elements (the 64-atom system's), where the Poisson fallback is
    within 6e-4 on the coarser mesh."""
    alpha, omega = coulomb_expansion()
    errs = []
    for n_el in (16, 37):
        fem = system.Fem1D(n_el, 0.0, 10.0)
        xq = fem.xq
        c, Q = 5.0 + 1e-3, 3.0
        g = np.exp(-(xq - c) ** 2)
        norm = Q / np.pi ** 1.5
        F = oracle.expansion_factor(alpha, xq, xq, fem.wJ, g[:, None])[:, :, 0]
        V = norm * np.einsum("t,ti,tj,tk->kji", omega, F, F, F, optimize=True)
        Z, Y, X = np.meshgrid(xq, xq, xq, indexing="ij")
        r = np.sqrt((X - c) ** 2 + (Y - c) ** 2 + (Z - c) ** 2)
        exact = Q * scipy.special.erf(r) / r
        errs.append(np.linalg.norm(V - exact) / np.linalg.norm(exact))
    assert errs[0] > 0.1 and errs[1] < 0.02


def test_linear_in_the_charge():
    fem, rho, _ = _gaussian_case(12)
    edges = [np.linspace(0, 10, 13)] * 3
    p1, _ = poisson.solve_hartree(rho, edges, [[3.0, 5.0, 5.0, 5.0]], n_outer=8)
    p2, _ = poisson.solve_hartree(2.0 * rho, edges, [[6.0, 5.0, 5.0, 5.0]], n_outer=8)
    assert np.abs(p2 - 2.0 * p1).max() < 1e-8 * np.abs(p2).max()


def test_exact_factor_integrals_remove_the_quadrature_error():
    """oracle.expansion_kernel_exact: the factor integrals by product
    integration (closed-form moments of each element's quadratic against
    exp(-alpha t^2)).  Along the line through a unit-width Gaussian charge on
    the 64-atom system's mesh (120 elements on 32 bohr): relative L2 error
    1.5e-6 against 7.2e-2 for the quadrature sums; and the kernel reproduces
    the quadrature sums exactly for quadratics, where both are exact."""
    alpha, omega = coulomb_expansion()
    fem = system.Fem1D(120, 0.0, 32.0)
    xq, edges = fem.xq, np.linspace(0.0, 32.0, 121)
    K = oracle.expansion_kernel_exact(alpha, xq, edges, xq)
    c, Q = 7.3, 3.0
    g = np.exp(-(xq - c) ** 2)
    j = np.argmin(np.abs(xq - c))
    r = np.sqrt((xq - c) ** 2 + 2 * (xq[j] - c) ** 2)
    exact = Q * scipy.special.erf(r) / r
    errs = {}
    for name, F in (("exact", np.einsum("tiq,q->ti", K, g)),
                    ("quadrature", oracle.expansion_factor(alpha, xq, xq, fem.wJ,
                                                           g[:, None])[:, :, 0])):
        V = Q / np.pi ** 1.5 * np.einsum("t,ti,t,t->i", omega, F, F[:, j], F[:, j])
        errs[name] = np.linalg.norm(V - exact) / np.linalg.norm(exact)
    assert errs["exact"] < 1e-5 and errs["quadrature"] > 1e-2
    # the widest terms (alpha -> 0): the kernel integrates a quadratic exactly,
    # as the 3-point rule does
    U = np.stack([np.ones_like(xq), xq, xq ** 2], axis=1)
    small = np.array([1e-9])
    Ke = oracle.expansion_kernel_exact(small, xq, edges, xq)[0] @ U
    Kq = oracle.expansion_factor(small, xq, xq, fem.wJ, U)[0]
    assert np.abs(Ke - Kq).max() < 1e-6 * np.abs(Kq).max()


def test_oracle_hartree_contraction_against_closed_form():
    """The oracle's Tucker contraction of the expansion (the checker of the
    device Hartree), fed exact factor integrals, reproduces the closed-form
    potential of the 2-atom superposition density on the full 3-D grid: a
    known answer for its axis order, weights and term sum (measured 6.2e-5
    relative L2; the quadrature sums on this 0.625-bohr mesh: 0.13)."""
    spec = system.small_spec(n_el=16, rank=8)
    s = system.build_system(spec)
    grids = [b.fem.xq for b in s.basis]
    rho = oracle.sad_density(s.atoms, grids, spec.z_val, 1.0)
    alpha, omega = coulomb_expansion()
    quad = [(b.fem.xq, b.fem.wJ) for b in s.basis]
    K = [oracle.expansion_kernel_exact(alpha, g, np.linspace(b.fem.x0, b.fem.x1, b.fem.n_el + 1), g)
         for g, b in zip(grids, s.basis)]
    U = [np.eye(g.size) for g in grids]
    V = oracle.hartree(alpha, omega, rho, quad, U, grids, kernels=K)
    Z, Y, X = np.meshgrid(grids[2], grids[1], grids[0], indexing="ij")
    exact = np.zeros_like(rho)
    for a in s.atoms:
        r = np.sqrt((X - a[0]) ** 2 + (Y - a[1]) ** 2 + (Z - a[2]) ** 2)
        exact += spec.z_val * scipy.special.erf(r) / r
    assert np.linalg.norm(V - exact) / np.linalg.norm(exact) < 1e-4
