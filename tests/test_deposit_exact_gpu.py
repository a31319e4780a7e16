"""Bit-exactness of the deposit's fixed-point accumulation.

The accumulate kernel sums every contribution as an int64 fixed-point value
q = round(w * phi_x * phi_y * phi_z * scale) (float32 products, power-of-two
scale fixed by max|w| max|phi|^3 and n).  Sparse tiles add q through two
32-bit shared-memory words (HI, LO), dense tiles through int64 atomics; both
must give the same integer per cell.  The float64 output is that integer
times 1/scale (exact), so it is compared bit for bit against the integers
rebuilt here in numpy from the same float32 arithmetic.  The catalogue has
a uniform part (tiles on the 32-bit path), a tight clump (tiles over the
32-bit bounds, int64 path) and negative weights (negative contributions)."""
import numpy as np
import pytest
import torch

from pyhermes_gb300 import kernels
from pyhermes_gb300.phi import sample_scaling_function

pytestmark = pytest.mark.gpu
PHI = sample_scaling_function()
RES = 1024


def _f32_up(v):
    """float32 rounded up (as __double2float_ru for v >= 0)."""
    f = np.float32(v)
    return np.nextafter(f, np.float32(np.inf)) if float(f) < v else f


def _f32_to_ll_rn(v):
    """Round-half-away int64 of float32 values from their bits (the
    kernel's integer conversion)."""
    b = v.view(np.int32).astype(np.int64)
    e = (b >> 23) & 0xFF
    m = (b & 0x7FFFFF) | 0x800000
    q = np.zeros_like(m)
    big = e >= 150
    q[big] = m[big] << (e[big] - 150)
    sh = 150 - e
    small = (~big) & (e != 0) & (sh < 25)
    q[small] = (m[small] + (np.int64(1) << (sh[small] - 1))) >> sh[small]
    return np.where(b < 0, -q, q)


def _exact_deposit(pos, w, J, box):
    L = 1 << J
    S = PHI.size // RES
    n = w.size
    wmax = _f32_up(np.abs(w).max())
    pmax = _f32_up(np.abs(PHI).max())
    bound = float(n) * float(wmax) * float(pmax) ** 3
    e = max(np.frexp(bound)[1], -60) if bound > 0 else -60
    scale = np.ldexp(1.0, 62 - e)
    s = pos * (L / box)
    c = np.floor(s)
    f = np.clip(((s - c) * RES).astype(np.int64), 0, RES - 1)
    c = c.astype(np.int64) & (L - 1)
    phif = PHI.astype(np.float32)
    wf = w.astype(np.float32)
    acc = np.zeros(L ** 3, dtype=np.int64)
    sf = np.float32(scale)
    for a in range(S):
        px = wf * phif[f[:, 0] + RES * a]
        for b in range(S):
            pxy = px * phif[f[:, 1] + RES * b]
            for cc in range(S):
                q = _f32_to_ll_rn((pxy * phif[f[:, 2] + RES * cc]) * sf)
                idx = (((c[:, 0] - a) & (L - 1)) * L + ((c[:, 1] - b) & (L - 1))) * L + ((c[:, 2] - cc) & (L - 1))
                np.add.at(acc, idx, q)
    return acc.astype(np.float64) * (1.0 / scale)


@pytest.mark.parametrize("seed", [0, 1])
def test_split_and_int64_tiles_are_bit_exact(seed):
    rng = np.random.default_rng(seed)
    J, box = 7, 1000.0
    n_u, n_c = 20_000, 5_000
    pos = np.concatenate([rng.uniform(0.0, box, (n_u, 3)),
                          np.mod(rng.normal(400.0, 6.0, (n_c, 3)), box)])
    w = rng.uniform(-0.5, 1.5, n_u + n_c)
    t = lambda a: torch.as_tensor(a, device="cuda")
    phi = t(PHI)
    eps64, _, _ = kernels.deposit(t(pos), t(w), J, box, phi, out_dtype=torch.float64)
    ref = _exact_deposit(pos, w, J, box)
    got = eps64.cpu().numpy().reshape(-1)
    assert np.array_equal(got, ref), (np.abs(got - ref).max(), np.abs(ref).max())
    # the float32 output is a function of the same integers: order-free, so a
    # permutation of the particles gives the same bits
    perm = rng.permutation(w.size)
    e1, _, _ = kernels.deposit(t(pos), t(w), J, box, phi)
    e2, _, _ = kernels.deposit(t(pos[perm]), t(w[perm]), J, box, phi)
    assert torch.equal(e1, e2)
    assert float((e1.double() - eps64).abs().max()) <= 2.0 ** -22 * float(eps64.abs().max())
