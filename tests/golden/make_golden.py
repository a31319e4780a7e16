"""Generates the golden fixtures in tests/golden/ by running the UNMODIFIED
PyHermes reference (read from a local checkout) under a minimal stub package
(``tests/golden/refshim``: numba -> plain Python, PyWavelets ->
scaling-function cascade, termcolor/json5/yaml stubs).

Usage:  python tests/golden/make_golden.py /path/to/PyHermes [section ...]

Fixtures are small (J <= 5) seeded cases.  The tests never import the
reference; they read these .npz files.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _setup(ref_root):
    sys.path[:0] = [os.path.join(HERE, "refshim"), ref_root, REPO]
    import logging

    logging.disable(logging.CRITICAL)


def _save(name, **arrays):
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, {k: getattr(v, "shape", None) for k, v in arrays.items()})


def gen_phi():
    from pyhermes.utils.corr3pcf_multipoles import cal_gamma
    from pyhermes.utils.wavelet_grid import fourier_power_spectrum, sample_scaling_function

    phi = sample_scaling_function("db2", 10)
    pw16 = fourier_power_spectrum(phi, 0, 1, 16, 1024)
    pw32_bw2 = fourier_power_spectrum(phi, 0, 2, 64, 1024)
    gamma = cal_gamma(phi, 3, 1024)
    _save("phi_db2", phi=phi, power_L16=pw16, power_L32_bw2=pw32_bw2, gamma=gamma)


def _projection(pos, J, weights=None, field_value=None, mode="catalog", box=1000.0):
    from pyhermes.base.sfc_projection import SFCProjection

    params = {"particle_pos": pos, "J": J, "box_size": box, "weight_normalization": mode}
    if weights is not None:
        params["catalog_weight"] = weights
    if field_value is not None:
        params["field_value"] = field_value
    task = SFCProjection({"SFCProjection": params})
    return task.run(save_result=False)


def gen_deposit():
    rng = np.random.default_rng(0)
    cases = {}
    # uniform, unit weights, catalog normalisation (the CPU-runnable config at small J)
    pos = rng.uniform(0.0, 1000.0, (2000, 3))
    f = _projection(pos, 4)
    cases["uniform_J4"] = (pos, np.ones(2000), np.ones(2000), "catalog", 4, f)
    # weighted + field values, 'field' normalisation, J=5, includes exact cell edges
    pos = rng.uniform(0.0, 1000.0, (3000, 3))
    pos[:10] = np.floor(pos[:10] / (1000.0 / 32)) * (1000.0 / 32)  # exactly on cell corners
    pos[10:20, 0] = 0.0
    pos[20:30, 1] = np.nextafter(1000.0, 0.0)
    w = rng.lognormal(0.0, 0.3, 3000)
    q = rng.uniform(0.5, 1.5, 3000)
    f = _projection(pos, 5, weights=w, field_value=q, mode="field")
    cases["weighted_J5"] = (pos, w, q, "field", 5, f)
    # raw normalisation, single particle
    pos = np.array([[123.456, 987.654, 0.001]])
    f = _projection(pos, 4, weights=np.array([2.5]), mode="raw")
    cases["single_raw_J4"] = (pos, np.array([2.5]), np.ones(1), "raw", 4, f)
    for name, (pos, w, q, mode, J, f) in cases.items():
        _save(f"deposit_{name}", pos=pos, catalog_weight=w, field_value=q, mode=np.array(mode),
              J=np.array(J), box=np.array(1000.0), epsilon=f.epsilon,
              field_integral=np.array(f.sfc_info["field_integral"]),
              catalog_weight_sum=np.array(f.sfc_info["catalog_weight_sum"]),
              raw_field_weighted_sum=np.array(f.sfc_info["raw_field_weighted_sum"]))


SECTIONS = {"phi": gen_phi, "deposit": gen_deposit}


def main(argv):
    if len(argv) < 2:
        print(__doc__)
        return 2
    _setup(argv[1])
    names = argv[2:] or list(SECTIONS)
    for n in names:
        SECTIONS[n]()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
