"""The tensor-core contraction (bin x bin product on tcgen05, BF16x3
operands) against the float64 oracle and the all-FP32 CUDA-core kernel.

Bounds: against the oracle, every S[b2, b3] within 2e-5 of the largest |S|
of the set (the FP32 fields and stencil set the floor, as for the FP32
kernel); tensor-core vs FP32 kernel within 1e-5 of the largest |S|, which is
the BF16x3 product's representation error (~2^-24 per operand) summed
over the cells.  Runs are bitwise reproducible.
"""
import numpy as np
import pytest
import torch

import oracle
from pyhermes_gb300 import multipole as mp
from pyhermes_gb300.phi import cal_gamma, sample_scaling_function
from pyhermes_gb300.window import phi_power_device, rfft_field

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()
GAM = cal_gamma(PHI, 3, 1024)


def _field(J, seed):
    rng = np.random.default_rng(seed)
    L = 1 << J
    n = 20 * L ** 3 // 8
    pos = rng.uniform(0.0, 1000.0, (n, 3))
    pos[: n // 3] = pos[: n // 3] * 0.3 + 350.0
    eps = oracle.deposit(pos, np.full(n, 1.0 / n), PHI, J, 1000.0)
    return eps - eps.mean()


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / np.abs(b).max()


def _engines(*args, **kw):
    return (mp.multipole_contract_engine(*args, engine="tensor", **kw),
            mp.multipole_contract_engine(*args, engine="simt", **kw))


def test_tensor_engine_matches_oracle_and_fp32_kernel():
    from scipy.fft import fftn, ifftn

    J, L = 5, 32
    eps = _field(J, 4)
    et = torch.as_tensor(eps, dtype=torch.float32, device="cuda")
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    l, m = 3, 1
    r2, r3 = [6.0, 8.5, 11.0], [7.0, 10.0]
    spec = rfft_field(et)
    f2 = mp.multipole_fields(spec, J, l, m, r2, P)
    f3 = mp.multipole_fields(spec, J, l, -m, r3, P)
    Pn = oracle.fourier_power(PHI, 1, L)
    s = fftn(eps)
    a2 = np.stack([ifftn(s * oracle.radial_multipole_window(L, Pn, r, l, m)) for r in r2])
    a3 = np.stack([ifftn(s * oracle.radial_multipole_window(L, Pn, r, l, -m)) for r in r3])
    ref = 4 * np.pi * oracle.contract_bins(eps, a2, a3, GAM) / L ** 3
    tc, simt = _engines(et, f2, 3, GAM, J, fields3=f3, nb3=2)
    status = mp.contract_status(J)
    assert status == 0, f"tensor-core kernel wait {status} gave up"
    assert _rel(tc, ref) < 2e-5, _rel(tc, ref)
    assert _rel(tc, simt) < 1e-5, _rel(tc, simt)
    # shared field and radii: a3 from the conjugate of a2's batch
    f2b = mp.multipole_fields(spec, J, l, -m, r2, P)
    ref_c = 4 * np.pi * oracle.contract_bins(
        eps, a2, np.stack([ifftn(s * oracle.radial_multipole_window(L, Pn, r, l, -m)) for r in r2]), GAM) / L ** 3
    tcc, simtc = _engines(et, f2, 3, GAM, J, conj_sign=(-1) ** ((l + m) % 2))
    assert _rel(tcc, ref_c) < 2e-5 and _rel(tcc, simtc) < 1e-5
    tce, _ = _engines(et, f2, 3, GAM, J, fields3=f2b, nb3=3)
    assert _rel(tcc, tce) < 1e-5
    # single-bin ([cell]) layouts on either side
    g2 = mp.multipole_fields(spec, J, l, m, [r2[1]], P)
    g3 = mp.multipole_fields(spec, J, l, -m, [r3[0]], P)
    t11, s11 = _engines(et, g2, 1, GAM, J, fields3=g3, nb3=1)
    assert abs(t11[0, 0] - ref[1, 0]) < 2e-5 * np.abs(ref).max() and abs(t11[0, 0] - s11[0, 0]) < 1e-5 * abs(s11[0, 0])
    t31, _ = _engines(et, f2, 3, GAM, J, fields3=g3, nb3=1)
    assert _rel(t31[:, 0], ref[:, 0]) < 2e-5
    t13, _ = _engines(et, g2, 1, GAM, J, fields3=f3, nb3=2)
    assert _rel(t13[0], ref[1]) < 2e-5


@pytest.mark.parametrize("J,chunk_x,ctas", [(6, 0, 0), (7, 32, 1), (7, 0, 2)])
def test_tensor_engine_many_bins_matches_fp32_kernel(J, chunk_x, ctas):
    """15 radii (the headline's bin count) at J = 6, 7 and several tile
    choices: tensor-core vs FP32 kernel, the status word clear, bitwise
    reproducible."""
    L = 1 << J
    g = torch.Generator(device="cuda").manual_seed(J)
    et = torch.randn((L, L, L), generator=g, device="cuda", dtype=torch.float32)
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    radii = list(np.linspace(1.0, 0.3 * L, 15))
    f = mp.multipole_fields(rfft_field(et), J, 4, 2, radii, P)
    kw = dict(conj_sign=1, chunk_x=chunk_x, ctas_per_sm=ctas)
    tc, simt = _engines(et, f, 15, GAM, J, **kw)
    assert mp.contract_status(J) == 0
    assert np.all(np.isfinite(tc))
    assert _rel(tc, simt) < 1e-5, _rel(tc, simt)
    tc2 = mp.multipole_contract_engine(et, f, 15, GAM, J, engine="tensor", **kw)
    assert np.array_equal(tc, tc2)


@pytest.mark.parametrize("J,chunk_x,ctas", [(6, 0, 0), (7, 32, 1)])
def test_bin_major_path_is_bit_identical(J, chunk_x, ctas):
    """Fields in the bin-major layout the inverse FFT writes (no interleave)
    hold the same values as the interleaved layout, and the tensor-core
    contraction reading them gives bit-identical S: shared field with 15 and
    with 1 radius, separate a3 fields with nb3 != nb2, and a3 of one radius."""
    L = 1 << J
    g = torch.Generator(device="cuda").manual_seed(100 + J)
    et = torch.randn((L, L, L), generator=g, device="cuda", dtype=torch.float32)
    P = phi_power_device(PHI, L, 1, 1024, "cuda")
    spec = rfft_field(et)
    radii = list(np.linspace(1.0, 0.3 * L, 15))
    l, m = 5, 3
    fi = mp.multipole_fields(spec, J, l, m, radii, P)
    fb = mp.multipole_fields(spec, J, l, m, radii, P, bin_major=True)
    assert fb.shape == (15, L ** 3)
    assert torch.equal(fb, fi[:, :15].t())
    kw = dict(chunk_x=chunk_x, ctas_per_sm=ctas)
    s_i = mp.multipole_contract_engine(et, fi, 15, GAM, J, conj_sign=-1, **kw)
    s_b = mp.multipole_contract_engine(et, fb, 15, GAM, J, conj_sign=-1, bin_major=True, **kw)
    assert mp.contract_status(J) == 0
    assert np.array_equal(s_i, s_b)
    r3 = radii[2:9]
    gi = mp.multipole_fields(spec, J, l, -m, r3, P)
    gb = mp.multipole_fields(spec, J, l, -m, r3, P, bin_major=True)
    s_i = mp.multipole_contract_engine(et, fi, 15, GAM, J, fields3=gi, nb3=7, **kw)
    s_b = mp.multipole_contract_engine(et, fb, 15, GAM, J, fields3=gb, nb3=7, bin_major=True, **kw)
    assert np.array_equal(s_i, s_b)
    h_i = mp.multipole_fields(spec, J, l, -m, [radii[4]], P)
    h_b = mp.multipole_fields(spec, J, l, -m, [radii[4]], P, bin_major=True)
    assert torch.equal(h_i, h_b)
    s_i = mp.multipole_contract_engine(et, fi, 15, GAM, J, fields3=h_i, nb3=1, **kw)
    s_b = mp.multipole_contract_engine(et, fb, 15, GAM, J, fields3=h_b, nb3=1, bin_major=True, **kw)
    assert np.array_equal(s_i, s_b)
    s_i = mp.multipole_contract_engine(et, h_i, 1, GAM, J, fields3=gi, nb3=7, **kw)
    s_b = mp.multipole_contract_engine(et, h_b, 1, GAM, J, fields3=gb, nb3=7, bin_major=True, **kw)
    assert np.array_equal(s_i, s_b)
    assert mp.contract_status(J) == 0
