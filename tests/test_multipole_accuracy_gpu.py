"""3PCF multipoles at the headline's ell range against float64 oracle
fixtures (tests/golden/make_multipole_fixtures.py), errors stated per sample
and per value.

* J=7, l = 0..10: the a_lm fields of every m at l = 10 against oracle
  fields computed here; DDD_l of delta = D - R and of R, and zeta_l, on a
  3x3 (r12, r13) thin-shell grid against multipole_grid_J7.npz, for both
  contraction engines.  The fields are the oracle's float64 deposits, so the
  comparison isolates the multipole path (float32 FFTs, windows, stencil).
* J=8 (the C3 unit): 1,000,000 lognormal points + 5,000,000 uniform randoms
  through SFCProjection -> Corr_3PCF_Multipole (GPU deposit included), one
  (r12, r13) sample, l = 0..10, against c3_unit_J8.npz.

Bounds, per (r12, r13) sample: |got_l - ref_l| <= bound * max_l' |ref_l'|,
the error of each multipole relative to the largest multipole of the same
sample (not of the whole set).  FP32 CUDA-core contraction ("simt") 1e-5;
BF16x3 tensor-core contraction ("tensor") 1e-4 (the bound stated for the
mixed-precision path).  The plain per-value relative error |got - ref| / |ref|
is printed beside it: it grows as a multipole falls below the sample's
leading one (a value 60x below carries the fields' FP32 rounding, ~7e-7 of
max |a_lm|, times 60).  Summands S_lm: relative to the largest |S| of their
(l, m) matrix, the same bounds.
"""
import os
import sys

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.phi import sample_scaling_function
from pyhermes_gb300.window import phi_power_device, rfft_field

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_multipole_fixtures as fx  # noqa: E402

PHI = sample_scaling_function()
BOUND = {"simt": 1e-5, "tensor": 1e-4}


def _per_value(got, ref):
    got, ref = np.asarray(got, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    return np.abs(got - ref) / np.abs(ref)


def _per_sample(got, ref):
    """|got - ref| over the largest |ref| of the same sample (last axis = l)."""
    got, ref = np.asarray(got, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    return np.abs(got - ref) / np.abs(ref).max(axis=-1, keepdims=True)


@pytest.fixture(scope="module")
def grid():
    g = np.load(os.path.join(HERE, "golden", "multipole_grid_J7.npz"))
    pos, w, rpos = fx.grid_catalogues(int(g["seed"]))
    ed, er = fx.catalog_fields(pos, w, rpos, int(g["J"]), PHI)
    return g, ed - er, er


def test_fields_l10_every_m_match_oracle(grid):
    from scipy.fft import fftn, ifftn

    g, delta, _ = grid
    J, L = int(g["J"]), 1 << int(g["J"])
    radii = [r * L / fx.BOX for r in g["radii"]]
    dt = torch.as_tensor(delta, dtype=torch.float32, device="cuda")
    spec = rfft_field(dt)
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    Pn = oracle.fourier_power(PHI, 1, L)
    s = fftn(delta, workers=os.cpu_count())
    worst = 0.0
    for m in range(-10, 11):
        f = mp.multipole_fields(spec, J, 10, m, radii, P).cpu().numpy()
        for b, r in enumerate(radii):
            ref = ifftn(s * oracle.radial_multipole_window(L, Pn, r, 10, m), workers=os.cpu_count()).ravel()
            err = np.abs(f[:, b] - ref).max() / np.abs(ref).max()
            worst = max(worst, err)
            assert err < 1e-5, (m, b, err)
    print(f"fields J=7 l=10 every m: max |delta a| / max |a| = {worst:.2e}")


@pytest.mark.parametrize("engine", ["simt", "tensor"])
def test_grid_ddd_and_zeta_match_oracle(grid, engine):
    g, delta, er = grid
    J = int(g["J"])
    radii = [float(r) for r in g["radii"]]
    pairs = [(a, b) for a in radii for b in radii]
    dt = torch.as_tensor(delta, dtype=torch.float32, device="cuda")
    rt = torch.as_tensor(er, dtype=torch.float32, device="cuda")
    n = len(radii)
    got = {}
    for name, f in (("delta", dt), ("random", rt)):
        eng = mp.MultipoleEngine(f, f, f, PHI, J, fx.BOX, engine=engine)
        got[name] = eng.ddd(pairs, 0, int(g["lmax"])).reshape(n, n, -1)
        # the summands of every m at l = 10 (S_lm of the shared-field engine)
        k0 = sum(l + 1 for l in range(10))
        for m in range(11):
            S = eng.summands(10, m, radii, radii)
            ref = g["S_" + name][k0 + m]
            err = np.abs(S - ref).max() / np.abs(ref).max()
            assert err < BOUND[engine], (engine, name, m, err)
    scale = ((1 << J) / fx.BOX) ** 9
    zeta, _, _ = mp.mixing_solve(got["delta"].reshape(n * n, -1) * scale, got["random"].reshape(n * n, -1) * scale,
                                 int(g["lmax"]))
    cases = {"ddd_delta": (got["delta"], g["ddd_delta"]), "ddd_random": (got["random"], g["ddd_random"]),
             "zeta": (zeta.reshape(n, n, -1), g["zeta"])}
    for k, (a, b) in cases.items():
        e, v = _per_sample(a, b), _per_value(a, b)
        print(f"{engine} J=7 3x3 grid l<=10 {k}: max err / sample max {e.max():.2e}; "
              f"per-value rel err max {v.max():.2e} median {np.median(v):.1e}")
    for k, (a, b) in cases.items():
        e = _per_sample(a, b)
        assert e.max() < BOUND[engine], (engine, k, e.max(), np.unravel_index(np.argmax(e), e.shape))


@pytest.mark.parametrize("engine", ["simt", "tensor"])
def test_c3_unit_J8_zeta_per_ell_matches_oracle(engine):
    """The C3 configuration's unit: 1M lognormal + 5M uniform randoms at
    J=8, delta = D - R, one (r12, r13) sample, l = 0..10, end to end through
    the public API (GPU deposit, fields, contraction, mixing solve)."""
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(os.path.join(HERE, "golden", "c3_unit_J8.npz"))
    seeds = dict(zip(("field", "poisson", "jitter", "weights", "random"), (int(v) for v in g["seeds"])))
    cells = fx.unit_cells_decode(int(g["cells_first"]), g["cells_diff"])
    pos, w, rpos = fx.unit_positions(cells, seeds, int(g["ng"]), int(g["n_rand"]))
    J = int(g["J"])
    d = SFCProjection({"SFCProjection": {"particle_pos": pos, "catalog_weight": w, "J": J,
                                         "box_size": fx.BOX}}).run(save_result=False)
    r = SFCProjection({"SFCProjection": {"particle_pos": rpos, "J": J, "box_size": fx.BOX}}).run(save_result=False)
    res = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": d, "random": r,
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [float(g["r12"])], "r13": [float(g["r13"])]},
        "l_min": 0, "l_max": int(g["lmax"]), "products": "zeta_l", "contraction_engine": engine}}).run(
        save_result=False)
    for k in ("delta_ddd_l", "rrr_l", "zeta_l"):
        e, v = _per_sample(getattr(res, k), g[k]), _per_value(getattr(res, k), g[k])
        print(f"{engine} C3 unit J=8 {k}: max err / sample max {e.max():.2e}; per-l rel err "
              f"{np.array2string(v.ravel(), precision=1)}")
    for k in ("delta_ddd_l", "rrr_l", "zeta_l"):
        e = _per_sample(getattr(res, k), g[k])
        assert e.max() < BOUND[engine], (engine, k, e.max(), int(np.argmax(e)))
