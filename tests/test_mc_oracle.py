"""Oracle Monte Carlo 3PCF against the reference's outputs (golden)."""
import os

import numpy as np

import oracle


def test_triangle_offsets_and_box_random_estimator(golden_dir):
    g = np.load(os.path.join(golden_dir, "mc3pcf_J4.npz"))
    params = [(0.3, 1.0, 0.2, 2.0), (-0.7, 4.0, -0.9, 0.5), (0.999, 0.1, 0.9999, 6.0)]
    for i, (m, p, c, a) in enumerate(params):
        np.testing.assert_allclose(oracle.generate_triangle_offsets(2.0, 3.5, m, p, c, a), g["offsets"][i],
                                   rtol=1e-14, atol=1e-15)
    phi = np.load(os.path.join(golden_dir, "phi_db2.npz"))["phi"]
    w = g["weights"]
    pw, _ = oracle.projection_weights(w, np.ones_like(w), "catalog")
    eps = oracle.deposit(g["pos"], pw, phi, 4, 1000.0)
    L = 16
    centers = np.random.default_rng(42 + 1000003).uniform(0.0, float(L), (600, 3))
    sf = L / 1000.0
    sf9 = sf ** 9
    rho = 1.0 / L ** 3
    for it, mu in enumerate(g["box_mu"]):
        d = oracle.mc_box_random(eps, eps, eps, 4, centers, 150 * sf, 250 * sf, mu, 3, 43, it, phi)
        np.testing.assert_allclose(d * sf9, g["box_ddd"][it], rtol=1e-12)
        dd = oracle.mc_box_random(eps - rho, eps - rho, eps - rho, 4, centers, 150 * sf, 250 * sf, mu, 3, 43, it, phi)
        np.testing.assert_allclose(dd * sf9, g["box_delta_ddd"][it], rtol=1e-10)
    np.testing.assert_allclose(g["box_rrr"], rho ** 3 * sf9, rtol=1e-12)


def test_mlp_oracle_gradient_by_finite_differences():
    rng = np.random.default_rng(0)
    dims = [4, 6, 5, 1]
    n = sum(a * b + b for a, b in zip(dims[:-1], dims[1:]))
    p = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((7, 4))
    t = rng.standard_normal(7)
    loss, g = oracle.mlp_mse_grad(p, dims, x, t)
    h = 1e-6
    for i in rng.choice(n, 12, replace=False):
        e = np.zeros(n)
        e[i] = h
        fd = (oracle.mlp_mse_grad(p + e, dims, x, t)[0] - oracle.mlp_mse_grad(p - e, dims, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) < 1e-7 * max(1.0, abs(fd))
