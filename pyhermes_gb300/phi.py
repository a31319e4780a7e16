"""Host-side scaling-function tables: the sampled db2 phi, its Fourier power
spectrum and the triple-overlap matrix Gamma.

These are tiny precomputes shared by every GPU kernel (3072 phi samples,
L+1 spectrum samples, a 3x3 matrix); they stay on the host in float64 and are
uploaded once per field.

* ``sample_scaling_function`` follows ``pyhermes/utils/wavelet_grid.py:10-14``,
  which calls PyWavelets ``Wavelet(name).wavefun(level)`` and drops the last
  sample.  PyWavelets is not a dependency here; its published algorithm for
  orthogonal wavelets is the cascade below: start from the single
  approximation coefficient ``2**(level/2)``, apply ``level`` full upsampling
  convolutions with the reconstruction low-pass filter (output length
  ``2*n + F - 2``), then frame the result as ``[0, c..., 0, 0]``.  For db2 at
  level 10 that is 3073 samples, 3072 after the drop, support 3.
* ``fourier_power_spectrum`` follows ``pyhermes/utils/wavelet_grid.py:94-118``:
  a direct DFT of the sampled phi at k = 0, 1/L, ..., bandwidth.
* ``cal_gamma`` follows ``pyhermes/utils/corr3pcf_multipoles.py:22-30``.
"""

import math

import numpy as np

# Daubechies orthonormal low-pass reconstruction filters, from their closed
# forms.  db1 is the Haar filter; db2 has the classic sqrt(3) form.
_SQ3 = math.sqrt(3.0)
_RS2 = 1.0 / (4.0 * math.sqrt(2.0))
_REC_LO = {
    "db1": np.array([1.0 / math.sqrt(2.0), 1.0 / math.sqrt(2.0)]),
    "haar": np.array([1.0 / math.sqrt(2.0), 1.0 / math.sqrt(2.0)]),
    "db2": np.array([(1.0 + _SQ3) * _RS2, (3.0 + _SQ3) * _RS2,
                     (3.0 - _SQ3) * _RS2, (1.0 - _SQ3) * _RS2]),
}


def reconstruction_lowpass(wavelet_name):
    """Return the reconstruction low-pass filter of a supported wavelet."""
    key = str(wavelet_name).strip().lower()
    if key not in _REC_LO:
        raise ValueError(
            f"Unsupported wavelet '{wavelet_name}'. Supported: {sorted(_REC_LO)}."
        )
    return _REC_LO[key].copy()


def scaling_cascade(wavelet_name="db2", level=10):
    """Full cascade output ``[0, c..., 0, 0]`` (PyWavelets ``wavefun`` phi)."""
    rec_lo = reconstruction_lowpass(wavelet_name)
    flen = rec_lo.size
    coeffs = np.array([math.sqrt(2.0) ** level], dtype=np.float64)
    for _ in range(int(level)):
        out = np.zeros(2 * coeffs.size + flen - 2, dtype=np.float64)
        for j in range(flen):
            out[j:j + 2 * coeffs.size:2] += coeffs * rec_lo[j]
        coeffs = out
    p = 2 ** int(level)
    output_length = (flen - 1) * p + 1
    keep_length = 1
    for _ in range(int(level)):
        keep_length = 2 * keep_length + (flen - 2)
    if output_length - keep_length - 2 < 0:
        output_length = keep_length + 2
    if keep_length < coeffs.size:
        left = (coeffs.size - keep_length) // 2
        coeffs = coeffs[left:left + keep_length]
    right = output_length - keep_length - 1
    return np.concatenate(([0.0], coeffs, np.zeros(right)))


def sample_scaling_function(wavelet_name="db2", level=10):
    """Sampled scaling function with the last sample dropped (float64)."""
    return scaling_cascade(wavelet_name, level)[:-1]


def fourier_power_spectrum(phi_array, k_max, k_count, phi_resolution):
    """|phi_hat(k)|^2 at k = n * k_max / k_count, n = 0..k_count (float64)."""
    phi_array = np.asarray(phi_array, dtype=np.float64)
    n = phi_array.shape[0]
    dx = (n / phi_resolution) / n
    dk = k_max / k_count
    x = np.arange(n) * dx
    k = np.arange(k_count + 1) * dk
    out = np.empty(k_count + 1, dtype=np.float64)
    step = 256
    for s in range(0, k_count + 1, step):
        arg = (-2.0 * np.pi * k[s:s + step])[:, None] * x[None, :]
        re = np.sum(phi_array * dx * np.cos(arg), axis=1)
        im = np.sum(phi_array * dx * np.sin(arg), axis=1)
        out[s:s + step] = re * re + im * im
    return out


def cal_gamma(phi_array, phi_support, phi_resolution):
    """Triple-overlap matrix Gamma[l1, l2] = sum phi*roll(phi,l1*res)*roll(phi,l2*res)/res."""
    phi_array = np.asarray(phi_array, dtype=np.float64)
    gamma = np.zeros((phi_support, phi_support))
    for l1 in range(phi_support):
        for l2 in range(phi_support):
            r1 = np.roll(phi_array, l1 * phi_resolution)
            r2 = np.roll(phi_array, l2 * phi_resolution)
            gamma[l1, l2] = np.sum(phi_array * r1 * r2) / phi_resolution
    return gamma
