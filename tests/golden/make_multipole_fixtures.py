"""Generates the float64 oracle fixtures for the multipole accuracy tests at
the headline's ell range (tests/test_multipole_accuracy_gpu.py):

* ``multipole_grid_J7.npz``: J=7, a clustered catalogue (uniform points plus
  Gaussian clumps, numpy only) and a uniform random catalogue, delta = D - R;
  a 3x3 (r12, r13) thin-shell grid, l = 0..10.  Holds the summands S_lm of
  delta (eps1 = a2 = a3 source = delta) and of R, DDD_l of both and zeta_l.
* ``c3_unit_J8.npz``: J=8, 1,000,000 lognormal-clustered points (weights
  lognormal(0, 0.3)) and 5,000,000 uniform randoms, one (r12, r13) sample,
  l = 0..10: delta_ddd_l, rrr_l, zeta_l as the multipole task reports them
  (catalog normalisation, physical rescale (L / box)^9).

Inputs regenerate bit-exactly from the stored seeds: positions come from
numpy's PCG64 streams (the lognormal catalogue from its stored cell indices
plus seeded in-cell jitter), the deposits are the oracle's float64 C
restatement (no contraction of multiply-add), so the tests rebuild the same
fields on any host.  The checker is the oracle (oracle/), itself pinned to
the reference's own outputs by tests/golden/make_golden.py.

Usage:  python tests/golden/make_multipole_fixtures.py [grid] [unit]
Runtime on 8 host cores: ~15 min (grid), ~50 min (unit).
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle")]

BOX = 1000.0
LMAX = 10

GRID_J = 7
GRID_RADII = [40.0, 70.0, 110.0]
GRID_SEED = 21

UNIT_J = 8
UNIT_NDATA = 1_000_000
UNIT_NRAND = 5_000_000
UNIT_NG = 256
UNIT_SAMPLE = (50.0, 90.0)
UNIT_SEEDS = {"field": 3, "poisson": 4, "jitter": 5, "weights": 6, "random": 7}


def grid_catalogues(seed=GRID_SEED, n_data=300_000, n_rand=1_000_000):
    """(data pos, data weights, random pos): uniform points with a third of
    them in 40 Gaussian clumps (sigma 15 Mpc/h, periodic), lognormal(0, 0.3)
    weights; uniform randoms.  numpy PCG64 only."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, BOX, (n_data, 3))
    n_cl = n_data // 3
    centres = rng.uniform(0.0, BOX, (40, 3))
    which = rng.integers(0, 40, n_cl)
    pos[:n_cl] = np.mod(centres[which] + rng.standard_normal((n_cl, 3)) * 15.0, BOX)
    pos = np.minimum(pos, np.nextafter(BOX, 0.0))
    w = rng.lognormal(0.0, 0.3, n_data)
    rpos = rng.uniform(0.0, BOX, (n_rand, 3))
    return pos, w, rpos


def unit_positions(cells, seeds=UNIT_SEEDS, ng=UNIT_NG, n_rand=UNIT_NRAND):
    """Data positions from the lognormal sample's cell indices plus seeded
    uniform in-cell jitter, lognormal(0, 0.3) weights, uniform randoms."""
    cells = np.asarray(cells, dtype=np.int64)
    ix, iy, iz = cells // (ng * ng), (cells // ng) % ng, cells % ng
    cell = BOX / ng
    jit = np.random.default_rng(seeds["jitter"]).random((cells.size, 3))
    pos = (np.stack([ix, iy, iz], axis=1).astype(np.float64) + jit) * cell
    pos = np.minimum(pos, np.nextafter(BOX, 0.0))
    w = np.random.default_rng(seeds["weights"]).lognormal(0.0, 0.3, cells.size)
    rpos = np.random.default_rng(seeds["random"]).uniform(0.0, BOX, (n_rand, 3))
    return pos, w, rpos


def unit_cells_encode(cells):
    s = np.sort(np.asarray(cells, dtype=np.int64))
    return s[0], np.diff(s).astype(np.uint32)


def unit_cells_decode(first, diffs):
    return np.concatenate([[first], first + np.cumsum(diffs.astype(np.int64))])


def catalog_fields(pos, w, rpos, J, phi):
    """Catalog-normalised float64 fields (field_integral 1): eps_D, eps_R."""
    import oracle

    ed = oracle.deposit(pos, w / np.sum(w, dtype=np.float64), phi, J, BOX)
    er = oracle.deposit(rpos, np.full(rpos.shape[0], 1.0 / rpos.shape[0]), phi, J, BOX)
    return ed, er


def zeta_from(ddd, rrr):
    import oracle

    out = np.zeros_like(ddd)
    for s in range(ddd.shape[0]):
        out[s] = oracle.solve_multipoles_from_ratio(ddd[s], rrr[s], ddd.shape[1] - 1)[0]
    return out


def gen_grid():
    import oracle
    from pyhermes_gb300.phi import sample_scaling_function

    phi = sample_scaling_function()
    pos, w, rpos = grid_catalogues()
    ed, er = catalog_fields(pos, w, rpos, GRID_J, phi)
    delta = ed - er
    t0 = time.time()
    ddd_d, s_d = oracle.calc_ddd_multipole_grid(delta, delta, delta, GRID_RADII, GRID_RADII, 0, LMAX, phi, box=BOX)
    print(f"grid delta done in {time.time() - t0:.0f} s", flush=True)
    ddd_r, s_r = oracle.calc_ddd_multipole_grid(er, er, er, GRID_RADII, GRID_RADII, 0, LMAX, phi, box=BOX)
    print(f"grid random done in {time.time() - t0:.0f} s", flush=True)
    n = len(GRID_RADII)
    zeta = zeta_from(ddd_d.reshape(n * n, -1), ddd_r.reshape(n * n, -1))
    np.savez_compressed(os.path.join(HERE, "multipole_grid_J7.npz"), J=GRID_J, radii=np.asarray(GRID_RADII),
                        seed=GRID_SEED, lmax=LMAX, S_delta=s_d, S_random=s_r, ddd_delta=ddd_d, ddd_random=ddd_r,
                        zeta=zeta.reshape(n, n, -1))
    print("wrote multipole_grid_J7.npz", flush=True)


def gen_unit():
    import torch

    import oracle
    from pyhermes_gb300 import synthetic
    from pyhermes_gb300.phi import sample_scaling_function

    phi = sample_scaling_function()
    sd = UNIT_SEEDS
    ng = UNIT_NG
    G = synthetic.gaussian_field(ng, BOX, sigma=1.0, seed=sd["field"], device="cpu")
    rho = torch.exp(G.double() - 0.5).reshape(-1)
    cdf = torch.cumsum(rho, 0)
    gen = torch.Generator(device="cpu")
    gen.manual_seed(sd["poisson"])
    u = torch.rand(UNIT_NDATA, generator=gen, dtype=torch.float64) * cdf[-1]
    cells = torch.searchsorted(cdf, u).clamp_max(ng ** 3 - 1).numpy()
    first, diffs = unit_cells_encode(cells)
    pos, w, rpos = unit_positions(unit_cells_decode(first, diffs))
    ed, er = catalog_fields(pos, w, rpos, UNIT_J, phi)
    delta = ed - er
    r12, r13 = UNIT_SAMPLE
    t0 = time.time()
    ddd_d, s_d = oracle.calc_ddd_multipole_grid(delta, delta, delta, [r12], [r13], 0, LMAX, phi, box=BOX)
    print(f"unit delta done in {time.time() - t0:.0f} s", flush=True)
    ddd_r, s_r = oracle.calc_ddd_multipole_grid(er, er, er, [r12], [r13], 0, LMAX, phi, box=BOX)
    print(f"unit random done in {time.time() - t0:.0f} s", flush=True)
    scale = ((1 << UNIT_J) / BOX) ** 9  # (scale_factor^3)^3, theory/corr3pcf_multipole.py:944-952
    dd = ddd_d[0, 0][None] * scale
    rr = ddd_r[0, 0][None] * scale
    zeta = zeta_from(dd, rr)
    np.savez_compressed(os.path.join(HERE, "c3_unit_J8.npz"), J=UNIT_J, ng=ng, cells_first=first, cells_diff=diffs,
                        seeds=np.asarray([sd[k] for k in ("field", "poisson", "jitter", "weights", "random")]),
                        n_rand=UNIT_NRAND, r12=r12, r13=r13, lmax=LMAX, S_delta=s_d[:, 0, 0], S_random=s_r[:, 0, 0],
                        delta_ddd_l=dd, rrr_l=rr, zeta_l=zeta)
    print("wrote c3_unit_J8.npz", flush=True)


if __name__ == "__main__":
    which = sys.argv[1:] or ["grid", "unit"]
    if "grid" in which:
        gen_grid()
    if "unit" in which:
        gen_unit()
