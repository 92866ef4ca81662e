"""CPU checks of the learned-guess oracle: gradient against finite
differences, descriptor invariances, the target fit."""
import numpy as np

from oracle import mlp


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    sizes = [5, 7, 6, 3]
    n = sum(i * o + o for i, o in zip(sizes[:-1], sizes[1:]))
    p = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((9, 5))
    t = rng.standard_normal((9, 3))
    loss, g = mlp.loss_and_grad(p, sizes, x, t)
    h = 1e-6
    fd = np.array([(mlp.loss_and_grad(p + h * e, sizes, x, t)[0]
                    - mlp.loss_and_grad(p - h * e, sizes, x, t)[0]) / (2 * h)
                   for e in np.eye(n)])
    assert np.abs(fd - g).max() < 1e-7 * max(1.0, np.abs(g).max())


def test_descriptors_invariant_and_cut_off():
    rng = np.random.default_rng(1)
    pos = rng.uniform(0, 10, (6, 3))
    d = mlp.descriptors(pos, 32, 0.5, 0.25, 4.0, 8.0)
    # translation and rotation invariance, permutation equivariance
    Q = np.linalg.qr(rng.standard_normal((3, 3)))[0]
    d2 = mlp.descriptors(pos @ Q.T + 3.0, 32, 0.5, 0.25, 4.0, 8.0)
    assert np.allclose(d, d2, atol=1e-12)
    perm = rng.permutation(6)
    assert np.allclose(mlp.descriptors(pos[perm], 32, 0.5, 0.25, 4.0, 8.0), d[perm])
    # an isolated atom (beyond the cutoff) has a zero descriptor
    far = np.vstack([pos, [[100.0, 100.0, 100.0]]])
    assert np.all(mlp.descriptors(far, 32, 0.5, 0.25, 4.0, 8.0)[-1] == 0.0)


def test_fit_targets_is_the_weighted_ridge_solution():
    """fit_targets (separable normal equations) against the dense weighted
    ridge least-squares solution on the grid."""
    from ttdft_public_gb300 import learned
    rng = np.random.default_rng(2)
    atoms = rng.uniform(3, 9, (3, 3))
    grids = [np.linspace(0, 12, 20 + 3 * d) for d in range(3)]
    weights = [np.full(g.size, g[1] - g[0]) for g in grids]
    rho = rng.standard_normal((grids[2].size, grids[1].size, grids[0].size))
    c = learned.fit_targets(atoms, grids, weights, rho)
    F = learned.correction_factors(atoms, grids)
    Phi = np.einsum("jx,jy,jz->zyxj", F[0], F[1], F[2]).reshape(-1, F[0].shape[0])
    W = np.einsum("z,y,x->zyx", weights[2], weights[1], weights[0]).reshape(-1)
    A = Phi.T @ (W[:, None] * Phi)
    A += learned.RIDGE * np.mean(np.diag(A)) * np.eye(A.shape[0])
    ref = np.linalg.solve(A, Phi.T @ (W * rho.reshape(-1)))
    assert np.abs(c.ravel() - ref).max() < 1e-6 * np.abs(ref).max()
