"""GPU Monte Carlo 3PCF (interpolation, triplet estimator, Corr_3PCF) against
the reference goldens / float64 oracle, the hand-written MLP kernels against
the float64 oracle, and the learned proposal against uniform MC.

Tolerances: interpolation 2e-6 of max|n|; DDD / RRR / xi / zeta / Q within
1e-5 relative to the largest |value| over mu; MLP gradients 1e-4 relative to
max|g| (float32 vs float64); bfloat16 inference within 2e-2 of float32.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import mc3pcf
from pyhermes_gb300.phi import sample_scaling_function

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()


def _rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return np.abs(a - b).max() / np.abs(b).max()


def test_interp_matches_oracle():
    rng = np.random.default_rng(1)
    J = 6
    pos = rng.uniform(0, 1000, (30000, 3))
    eps = oracle.deposit(pos, np.full(30000, 1.0 / 30000), PHI, J, 1000.0)
    pts = rng.uniform(0, 64, (5000, 3))
    g = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    phi_t = torch.as_tensor(PHI, device="cuda")
    for off in [(0.0, 0.0, 0.0), (1.25, -3.5, 70.0)]:
        got = mc3pcf.interp(g, J, pts, phi_t, off).cpu().numpy()
        ref = oracle.interp(pts, eps, PHI, J, offset=off)
        assert _rel(got, ref) < 2e-6


def test_corr3pcf_box_random_matches_reference(golden_dir):
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "mc3pcf_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "box_random",
        "n_box_centers": 600, "base_seed": 42, "products": ["Q", "ddd"]}}).run()
    for k in ("ddd", "rrr", "delta_ddd", "xi12", "xi13", "xi23", "zeta", "zeta_H", "Q"):
        assert _rel(getattr(d, k), g["box_" + k]) < 1e-5, (k, getattr(d, k), g["box_" + k])


def test_corr3pcf_particle_centres_match_reference(golden_dir):
    """center='particle' against the reference: explicit random centres
    (ddd, rrr, d_delta_dd, r_delta_dd, delta_ddd) and the uniform-random
    shortcut r_delta_dd = rrr xi23 (with xi23 and zeta)."""
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "mc3pcf_particle_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    common = {"sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
              "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "particle", "base_seed": 7,
              "particle_pos1": g["cpos"], "particle_weight1": g["cw"]}
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": dict(common, random_pos1=g["rpos"], random_weight1=g["rw"],
                                            products=["ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"])}).run()
    for k in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd"):
        assert _rel(getattr(d, k), g["rpos_" + k]) < 1e-5, (k, getattr(d, k), g["rpos_" + k])
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": dict(common, products=["zeta", "ddd"])}).run()
    for k in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd", "xi23", "zeta"):
        assert _rel(getattr(d, k), g["uni_" + k]) < 1e-5, (k, getattr(d, k), g["uni_" + k])


def test_corr3pcf_vertex_windows_match_reference(golden_dir):
    """A shared gaussian window and a sphere on vertex 3 (particle centres,
    uniform random): ddd, rrr, deltas, xi23 and zeta."""
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "mc3pcf_particle_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": {
        "sfc_field": f, "random": "uniform", "r12": 150.0, "r13": 250.0, "angle_param": "mu",
        "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "particle", "base_seed": 7,
        "particle_pos1": g["cpos"], "particle_weight1": g["cw"],
        "window": {"type": "gaussian", "len_args": {"R": 40.0}},
        "window3": {"type": "sphere", "len_args": {"R": 60.0}}, "products": ["zeta", "ddd"]}}).run()
    for k in ("ddd", "rrr", "d_delta_dd", "r_delta_dd", "delta_ddd", "xi23", "zeta"):
        assert _rel(getattr(d, k), g["win_" + k]) < 1e-4, k


@pytest.mark.parametrize("case", ["fields", "uni1"])
def test_corr3pcf_random_fields_match_reference(golden_dir, case):
    """Random catalogues as fields: rrr by Monte Carlo over three random
    fields, or rho1 RR23(r23) with a uniform vertex 1."""
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(golden_dir, "mc3pcf_randoms_J4.npz"))
    f = SFCProjection({"SFCProjection": {"particle_pos": g["pos"], "catalog_weight": g["weights"], "J": 4,
                                         "box_size": 1000.0}}).run(save_result=False)
    r = SFCProjection({"SFCProjection": {"particle_pos": g["rpos"], "J": 4, "box_size": 1000.0}}).run(
        save_result=False)
    params = {"sfc_field": f, "r12": 150.0, "r13": 250.0, "angle_param": "mu",
              "mu": {"mu_min": -0.8, "mu_max": 0.8, "n_mu": 3}, "n_rot": 3, "center": "box_random",
              "n_box_centers": 600, "base_seed": 42}
    if case == "fields":
        params.update(random=r, products=["zeta", "ddd"])
        keys = ("ddd", "delta_ddd", "rrr", "zeta")
    else:
        params.update(random1="uniform", random2=r, random3=r, products=["zeta"])
        keys = ("delta_ddd", "rrr", "zeta")
    d = mc3pcf.Corr_3PCF({"Corr_3PCF": params}).run()
    for k in keys:
        assert _rel(getattr(d, k), g[f"{case}_{k}"]) < 1e-5, (k, getattr(d, k), g[f"{case}_{k}"])


def test_mlp_gradients_match_oracle():
    dims = [4, 128, 128, 128, 1]
    net = mc3pcf.MLP(dims, seed=3)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((1000, 4)).astype(np.float32)
    t = rng.standard_normal(1000).astype(np.float32)
    loss, g = net.grads(torch.as_tensor(x, device="cuda"), torch.as_tensor(t, device="cuda"))
    p = net.params.double().cpu().numpy()
    ref_loss, ref_g = oracle.mlp_mse_grad(p, dims, x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - ref_loss) < 1e-5 * max(1.0, ref_loss)
    assert _rel(g.cpu().numpy(), ref_g) < 1e-4
    y32 = net.forward(torch.as_tensor(x, device="cuda")).cpu().numpy().ravel()
    y16 = net.forward(torch.as_tensor(x, device="cuda"), bf16=True).cpu().numpy().ravel()
    yref = oracle.mlp_forward(p, dims, x.astype(np.float64))[-1].ravel()
    assert _rel(y32, yref) < 1e-5
    assert _rel(y16, yref) < 2e-2


@pytest.mark.parametrize("dims,batch", [([6, 128, 128, 128, 1], 50_000), ([4, 128, 128, 1], 1000),
                                        ([16, 128, 128, 128, 128, 128, 1], 128 * 152 * 3 + 77)])
def test_mlp_tensor_core_inference_matches_oracle(dims, batch):
    """hermes_mlp_infer_tc (hidden 128 x 128 layers on tcgen05, BF16 weights
    and activations) against the float64 oracle forward: within 2e-2 of the
    largest |y| (the BF16 rounding of weights and activations), several
    tiles per CTA and a ragged last tile."""
    net = mc3pcf.MLP(dims, seed=4)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((batch, dims[0])).astype(np.float32)
    ytc = net.infer(torch.as_tensor(x, device="cuda")).cpu().numpy()
    p = net.params.double().cpu().numpy()
    yref = oracle.mlp_forward(p, dims, x.astype(np.float64))[-1].ravel()
    assert ytc.shape == (batch,)
    assert _rel(ytc, yref) < 2e-2, _rel(ytc, yref)
    assert np.array_equal(ytc, net.infer(torch.as_tensor(x, device="cuda")).cpu().numpy())


def test_poisson_deviance_gradient_matches_numpy():
    """hermes_poisson_grad: loss = mean(exp(y) - t y), dy = (exp(y) - t)/n
    against float64 numpy."""
    import ctypes

    from pyhermes_gb300 import _lib
    from pyhermes_gb300.kernels import _ptr, _stream_ptr

    rng = np.random.default_rng(8)
    n = 100_003
    y = rng.normal(0.0, 1.5, n).astype(np.float32)
    t = rng.gamma(0.5, 2.0, n).astype(np.float32)
    yt, tt = torch.as_tensor(y, device="cuda"), torch.as_tensor(t, device="cuda")
    dy = torch.empty_like(yt)
    loss = ctypes.c_double(0.0)
    scratch = torch.empty(1, dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().hermes_poisson_grad(_ptr(yt), _ptr(tt), n, _ptr(dy), ctypes.byref(loss), _ptr(scratch),
                                                _stream_ptr(yt.device)), "poisson_grad")
    yd, td = y.astype(np.float64), t.astype(np.float64)
    assert abs(loss.value - np.mean(np.exp(yd) - td * yd)) < 1e-6 * np.mean(np.exp(yd))
    assert _rel(dy.cpu().numpy(), (np.exp(yd) - td) / n) < 1e-5


def test_mlp_training_reduces_loss():
    net = mc3pcf.MLP([4, 64, 64, 1], seed=1)
    rng = np.random.default_rng(5)
    x = torch.as_tensor(rng.uniform(-1, 1, (65536, 4)), dtype=torch.float32, device="cuda")
    t = torch.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2]
    losses = net.train(x, t, epochs=6, batch=4096, lr=3e-3)
    assert losses[-1] < 0.2 * losses[0]


def test_learned_proposal_is_unbiased_and_reduces_variance():
    """Clustered J=7 field: the learned proposal's weighted estimator agrees
    with uniform MC and has a smaller per-sample variance."""
    from pyhermes_gb300 import kernels, synthetic

    J, L = 7, 128
    pos, w = synthetic.lognormal_catalogue(200_000, sigma_g=1.5, ng=128)
    pw = torch.as_tensor(w / w.sum(), device="cuda")
    eps, _, _ = kernels.deposit(torch.as_tensor(pos, device="cuda"), pw, J, 1000.0,
                                torch.as_tensor(PHI, device="cuda"))
    rho = 1.0 / L ** 3
    lp = mc3pcf.LearnedProposal(eps, eps, eps, J, PHI, rho)
    configs = [(r1, r2, mu) for r1 in (1.5, 3.0) for r2 in (2.5, 5.0) for mu in (-0.5, 0.5)]
    losses = lp.train(configs, n_centers=100_000, n_rot_train=8, epochs=3, n_rot_eval=1)
    assert losses[-1] < losses[0]
    pool = torch.as_tensor(np.random.default_rng(9).uniform(0, L, (400_000, 3)), device="cuda")
    K = 400_000
    # centres with n1 = 0 contribute exactly 0: no mass there, mass everywhere else
    q = lp.proposal(pool, 2.0, 4.0, 0.3)
    _, n1 = lp.features(pool, 2.0, 4.0, 0.3, return_n1=True)
    assert float(q[n1 == 0].abs().sum()) == 0.0 and bool((q[n1 != 0] > 0).all())
    assert abs(float(q.sum()) - 1.0) < 1e-9
    est_u, vu = lp.estimate(pool, 2.0, 4.0, 0.3, K, seed=11, uniform=True)
    est_l, vl = lp.estimate(pool, 2.0, 4.0, 0.3, K, seed=12)
    var_u, var_l = float(vu.var()), float(vl.var())
    se = np.sqrt(var_u / K + var_l / K)
    assert abs(est_l - est_u) < 5 * se
    assert var_l < var_u / 1.5, (var_u, var_l)


def test_mc_sample_matches_interp_path_and_draws_unbiased_rotations():
    """hermes_mc_sample against three hermes_interp gathers for the same
    (centre, offset) pairs (sums to 1e-5); its on-device rotations give the
    same uniform-MC mean as host rotations (within 5 sigma); the learned
    proposal through it stays unbiased with a smaller variance per sample."""
    from pyhermes_gb300 import kernels, synthetic

    J, L = 7, 128
    pos, w = synthetic.lognormal_catalogue(200_000, sigma_g=1.5, ng=128)
    pw = torch.as_tensor(w / w.sum(), device="cuda")
    eps, _, _ = kernels.deposit(torch.as_tensor(pos, device="cuda"), pw, J, 1000.0,
                                torch.as_tensor(PHI, device="cuda"))
    rho = 1.0 / L ** 3
    lp = mc3pcf.LearnedProposal(eps, eps, eps, J, PHI, rho)
    rng = np.random.default_rng(5)
    pool = torch.as_tensor(rng.uniform(0, L, (300_000, 3)), device="cuda")
    n = 200_000
    idx = torch.as_tensor(rng.integers(0, pool.shape[0], n), device="cuda")
    wts = torch.as_tensor(rng.uniform(0.5, 1.5, n), device="cuda")
    off = torch.as_tensor(mc3pcf.rotation_offsets(2.0, 4.0, 0.3, n, rng=np.random.RandomState(3)), device="cuda")
    a, b = mc3pcf.mc_sample(lp.e1, lp.e2, lp.e3, J, pool, lp.phi_t, 2.0, 4.0, 0.3, n, idx=idx, weights=wts,
                            offsets=off)
    f = lp._f_pairs(pool[idx], off.cpu().numpy()) * wts
    assert abs(a - float(f.sum())) < 1e-5 * float(f.abs().sum())
    assert abs(b - float((f * f).sum())) < 1e-5 * float((f * f).sum())
    # device rotations vs host rotations (uniform MC, same pool)
    K = 400_000
    m_dev, se_dev, v_dev = lp.sample_stats(pool, 2.0, 4.0, 0.3, K, seed=21, uniform=True)
    m_host, vh = lp.estimate(pool, 2.0, 4.0, 0.3, K, seed=22, uniform=True)
    se = np.sqrt(se_dev ** 2 + float(vh.var()) / K)
    assert abs(m_dev - m_host) < 5 * se, (m_dev, m_host, se)
    # learned proposal through the fused kernel: unbiased, smaller estimator variance
    configs = [(r1, r2, mu) for r1 in (1.5, 3.0) for r2 in (2.5, 5.0) for mu in (-0.5, 0.5)]
    lp.train(configs, n_centers=100_000, n_rot_train=8, epochs=3, n_rot_eval=1)
    m_l, se_l, v_l = lp.sample_stats(pool, 2.0, 4.0, 0.3, K, seed=23)
    se = np.sqrt(se_dev ** 2 + se_l ** 2)
    assert abs(m_l - m_dev) < 5 * se, (m_l, m_dev, se)
    # variance per sample: the products of three lognormal densities are
    # heavy-tailed, so compare the median of 16 per-replicate variances
    q = lp.proposal(pool, 2.0, 4.0, 0.3)
    g = torch.Generator(device="cuda").manual_seed(24)
    vu, vl = [], []
    for r in range(16):
        nr = 50_000
        a, b = mc3pcf.mc_sample(lp.e1, lp.e2, lp.e3, J, pool, lp.phi_t, 2.0, 4.0, 0.3, nr, 1000 + r)
        vu.append(b / nr - (a / nr) ** 2)
        idx, wl = lp.draw(q, nr, g)
        a, b = mc3pcf.mc_sample(lp.e1, lp.e2, lp.e3, J, pool, lp.phi_t, 2.0, 4.0, 0.3, nr, 2000 + r, idx=idx,
                                weights=wl)
        vl.append(b / nr - (a / nr) ** 2)
    assert np.median(vl) < np.median(vu) / 1.5, (np.median(vu), np.median(vl))
    # centres x rotations with importance-sampled centres (fresh pools): unbiased
    mc_u, se_cu = lp.centre_estimate(2.0, 4.0, 0.3, 20_000, 32, seed=31, uniform=True)
    mc_l, se_cl = lp.centre_estimate(2.0, 4.0, 0.3, 20_000, 32, seed=32)
    assert abs(mc_l - mc_u) < 5 * np.sqrt(se_cu ** 2 + se_cl ** 2), (mc_u, mc_l, se_cu, se_cl)


@pytest.mark.parametrize("J", [4, 7])
def test_brick_layout_gathers_are_bit_identical(J):
    """hermes_field_to_bricks puts cell (x, y, z) at brick (x/2, y/2, z/2),
    slot (x%2, y%2, z%2); the brick-layout triplet and single-sample kernels
    read the same float32 values in the same order, so their float64 sums and
    per-triplet products equal the C-order kernels' exactly."""
    L = 1 << J
    g = torch.Generator(device="cuda").manual_seed(J)
    eps = [torch.rand((L, L, L), generator=g, device="cuda", dtype=torch.float32) for _ in range(3)]
    bricks = mc3pcf.field_bricks(eps[1], J)
    want = eps[1].view(L // 2, 2, L // 2, 2, L // 2, 2).permute(0, 2, 4, 1, 3, 5).reshape(-1)
    assert torch.equal(bricks, want)
    assert mc3pcf.field_bricks(eps[1], J) is bricks  # cached
    rng = np.random.default_rng(J)
    phi_t = torch.as_tensor(PHI, device="cuda")
    centres = torch.as_tensor(rng.uniform(0.0, L, (5000, 3)), device="cuda")
    off = mc3pcf.rotation_offsets(0.2 * L, 0.3 * L, 0.4, 7, rng=np.random.RandomState(J))
    for e1 in (eps[0], None):
        a, sa = mc3pcf.triplet_sum(e1, eps[1], eps[2], J, centres, off, phi_t, rho1=1.5, samples=True, bricks=False)
        b, sb = mc3pcf.triplet_sum(e1, eps[1], eps[2], J, centres, off, phi_t, rho1=1.5, samples=True, bricks=True)
        assert a == b
        assert torch.equal(sa, sb)
    a = mc3pcf.mc_sample(eps[0], eps[1], eps[2], J, centres, phi_t, 0.2 * L, 0.3 * L, 0.4, 20000, seed=9,
                         bricks=False)
    b = mc3pcf.mc_sample(eps[0], eps[1], eps[2], J, centres, phi_t, 0.2 * L, 0.3 * L, 0.4, 20000, seed=9,
                         bricks=True)
    assert a == b


def test_interp_indices_follow_the_reference_at_boundaries():
    """hermes_interp gathers the 27 cells around floor(s) with the phi samples
    at int((s - floor(s)) * res), both in the reference's float64 arithmetic
    (the kernel reads them from the float64 bits of s when 0 <= s < 2^30).
    Against a float64 restatement, for coordinates on and beside cell and
    sample boundaries, tiny, negative (offset) and ordinary ones: a cell or
    sample index off by one would move a value by ~1e-3 or more, far above
    the float32 tolerance of 2e-6."""
    J, L, res = 5, 32, 1024
    rng = np.random.default_rng(3)
    grid = rng.standard_normal((L, L, L)).astype(np.float32)
    phis = np.asarray(PHI, dtype=np.float32).astype(np.float64)
    k = np.arange(0, 4 * res)
    edge = np.concatenate([k / res, np.nextafter(k / res, 0.0), np.nextafter(k / res, 1e9)])[:3000]
    pos = np.stack([rng.uniform(0.0, L, 6000), rng.uniform(0.0, L, 6000), rng.uniform(0.0, L, 6000)], axis=1)
    pos[:3000, 0] = edge
    pos[3000:3100, 1] = rng.uniform(0.0, 1e-9, 100)
    pos[3100:3200] = np.floor(pos[3100:3200])
    off = (-7.25, 0.5, -0.3)  # makes some coordinates negative
    got = mc3pcf.interp(torch.as_tensor(grid, device="cuda"), J, torch.as_tensor(pos, device="cuda"),
                        torch.as_tensor(PHI, device="cuda"), offset=off).cpu().numpy()
    s = pos + np.asarray(off)
    c = np.floor(s).astype(np.int64)
    f = np.clip(((s - np.floor(s)) * res).astype(np.int64), 0, res - 1)
    g64 = grid.astype(np.float64)
    want = np.zeros(len(pos))
    for a in range(3):
        px = phis[f[:, 0] + a * res]
        for b in range(3):
            py = phis[f[:, 1] + b * res]
            for cc in range(3):
                v = g64[(c[:, 0] - a) % L, (c[:, 1] - b) % L, (c[:, 2] - cc) % L]
                want += v * px * py * phis[f[:, 2] + cc * res]
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-6)
