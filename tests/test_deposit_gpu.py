"""GPU deposit (hermes_deposit through the C ABI) against the float64 oracle.

Tolerance (float32 field vs float64 oracle): every cell within
2e-6 * max|eps| and relative L2 error <= 1e-6; the integer per-cell counts
are bit-exact; the field is bitwise reproducible across runs and particle
orderings (fixed-point accumulation).
"""
import os

import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import kernels, synthetic
from pyhermes_gb300.phi import sample_scaling_function

pytestmark = pytest.mark.gpu

PHI = sample_scaling_function()


def _gpu_deposit(pos, w, J, box=1000.0, out_dtype=torch.float32, counts=False):
    pos_t = torch.as_tensor(pos, dtype=torch.float64, device="cuda")
    w_t = torch.as_tensor(w, dtype=torch.float64, device="cuda")
    phi_t = torch.as_tensor(PHI, dtype=torch.float64, device="cuda")
    eps, cnt, ws = kernels.deposit(pos_t, w_t, J, box, phi_t, out_dtype=out_dtype, counts=counts)
    torch.cuda.synchronize()
    return eps, cnt, ws


def _assert_close(eps_gpu, ref, tol_inf=2e-6, tol_l2=1e-6):
    e = eps_gpu.double().cpu().numpy()
    scale = np.max(np.abs(ref))
    err = np.abs(e - ref)
    assert err.max() <= tol_inf * scale, (err.max(), scale)
    assert np.linalg.norm(e - ref) <= tol_l2 * np.linalg.norm(ref)


@pytest.mark.parametrize("name", ["uniform_J4", "weighted_J5", "single_raw_J4"])
def test_deposit_matches_reference_golden(golden_dir, name):
    d = np.load(os.path.join(golden_dir, f"deposit_{name}.npz"))
    pw, _ = oracle.projection_weights(d["catalog_weight"], d["field_value"], str(d["mode"]))
    eps, cnt, _ = _gpu_deposit(d["pos"], pw, int(d["J"]), counts=True)
    _assert_close(eps, d["epsilon"])
    ref_cnt = oracle.cell_counts(d["pos"], int(d["J"]), 1000.0)
    np.testing.assert_array_equal(cnt.cpu().numpy().astype(np.uint32), ref_cnt)


def test_deposit_cpu_config_200k_J7():
    pos = synthetic.uniform_catalogue(200_000, seed=0)
    w = np.full(200_000, 1.0 / 200_000)
    ref = oracle.deposit(pos, w, PHI, 7, 1000.0)
    eps, cnt, _ = _gpu_deposit(pos, w, 7, counts=True)
    _assert_close(eps, ref)
    np.testing.assert_array_equal(cnt.cpu().numpy().astype(np.uint32), oracle.cell_counts(pos, 7, 1000.0))
    eps64, _, _ = _gpu_deposit(pos, w, 7, out_dtype=torch.float64)
    _assert_close(eps64, ref, tol_inf=1e-6, tol_l2=5e-7)


def test_deposit_full_size_lognormal_J9():
    """4M clustered points at J=9: float32 field vs float64 oracle, integral
    conservation, and bitwise determinism under reordering."""
    pos, w = synthetic.lognormal_catalogue(4_000_000)
    pw = w / w.sum()
    ref = oracle.deposit(pos, pw, PHI, 9, 1000.0)
    eps, cnt, _ = _gpu_deposit(pos, pw, 9, counts=True)
    _assert_close(eps, ref)
    assert int(cnt.sum().item()) == 4_000_000
    assert abs(eps.double().sum().item() - 1.0) < 1e-5
    perm = np.random.default_rng(5).permutation(pos.shape[0])
    eps2, _, _ = _gpu_deposit(pos[perm], pw[perm], 9)
    assert torch.equal(eps, eps2)


def test_deposit_edge_cases():
    # empty catalogue -> zero field
    eps, cnt, _ = _gpu_deposit(np.zeros((0, 3)), np.zeros(0), 5, counts=True)
    assert float(eps.abs().max()) == 0.0 and int(cnt.sum()) == 0
    # points exactly on the box faces, corners and periodic wrap
    pos = np.array([[0.0, 0.0, 0.0], [np.nextafter(1000.0, 0), 0.0, 500.0],
                    [999.9999, 999.9999, 999.9999], [31.25, 62.5, 93.75]])
    w = np.array([1.0, 2.0, -0.5, 3.0])
    ref = oracle.deposit(pos, w, PHI, 5, 1000.0)
    eps, cnt, _ = _gpu_deposit(pos, w, 5, counts=True)
    _assert_close(eps, ref)
    np.testing.assert_array_equal(cnt.cpu().numpy().astype(np.uint32), oracle.cell_counts(pos, 5, 1000.0))


def test_deposit_rejects_nonfinite():
    pos = np.array([[1.0, 2.0, 3.0], [np.nan, 1.0, 1.0], [5.0, np.inf, 1.0]])
    w = np.ones(3)
    eps, _, ws = _gpu_deposit(pos, w, 4)
    assert kernels.deposit_rejected(ws) == 2
    ref = oracle.deposit(pos[:1], w[:1], PHI, 4, 1000.0)
    _assert_close(eps, ref)


def test_projection_api_matches_reference(golden_dir):
    from pyhermes_gb300.projection import SFCProjection

    d = np.load(os.path.join(golden_dir, "deposit_weighted_J5.npz"))
    task = SFCProjection({"SFCProjection": {
        "particle_pos": d["pos"], "catalog_weight": d["catalog_weight"], "field_value": d["field_value"],
        "weight_normalization": "field", "J": 5, "box_size": 1000.0}})
    f = task.run(save_result=False)
    assert f.field_integral == float(d["field_integral"])
    assert f.catalog_weight_sum == float(d["catalog_weight_sum"])
    assert f.field_kind == "catalog_field" and f.L == 32 and f.V == 32 ** 3
    _assert_close(f.epsilon_device, d["epsilon"])
