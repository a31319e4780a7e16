"""Batched execution of many catalogues of uneven size and J.

Each catalogue runs the same chain as the public API used one at a time:
``SFCProjection`` deposit, ``Corr_2PCF`` of the Gaussian-smoothed field
(``window`` = gaussian R, thick-shell bins, random = 'uniform') and
``Corr_3PCF_Multipole`` (thin shells on both sides, grid sampling,
random = 'uniform', products delta_ddd_l, rrr_l, zeta_l).  The public task
objects still do the host-side set-up (normalisation, smoothing, binning
windows, analytic RRR, mixing solve), so the results are the same numbers;
what is batched is the GPU work:

* catalogues are grouped by J; one set of 2PCF bin windows and one
  multipole engine (fixed device buffers, one captured graph) serve a whole
  group;
* the 2PCF pair products of up to four catalogues run in one pass over
  their spectra (``hermes_pair_products`` with four pairs);
* the multipole (l, m) loop -- rFFT, then for every (l, m) the radial
  multipole fields and the contraction -- is one CUDA graph per J
  (``GraphedMultipole``), replayed per catalogue with no host round trip
  inside; its contraction tile (x-chunk, CTAs per SM) comes from
  ``autotune.tune_contract``;
* the deposit tile of each J is tuned on the group's first catalogue
  (``autotune.tune_deposit``; the field does not depend on it).

``run_one_at_a_time`` is the unbatched path through the public classes.
``c4_catalogues`` builds the uneven catalogue set (sizes log-uniform in
[1e4, 2e6], odd seeds uniform and even seeds lognormal, J in {7, 8, 9} and
R in {5, 10, 20} Mpc/h round-robin).
"""

import math
import time

import numpy as np
import torch

from . import autotune, kernels, synthetic
from . import multipole as mp
from .corr2pcf import Corr_2PCF
from .projection import SFCProjection
from .window import pair_products, rfft_field


def c4_catalogues(n_cat=64, n_min=1e4, n_max=2e6, box=1000.0, device="cuda", js=(7, 8, 9), rs=(5.0, 10.0, 20.0)):
    """The uneven catalogue set: list of dicts (pos, weights, J, R, seed)."""
    cats = []
    lo, hi = math.log(n_min), math.log(n_max)
    for i in range(n_cat):
        seed = i + 1
        rng = np.random.default_rng(1000 + seed)
        n = int(round(math.exp(rng.uniform(lo, hi))))
        if seed % 2 == 1:
            pos = synthetic.uniform_catalogue(n, box=box, seed=seed)
            w = np.ones(n)
        else:
            pos, w = synthetic.lognormal_catalogue(n, box=box, seed_field=seed, seed_poisson=seed + 100,
                                                   seed_weights=seed + 200, device=device)
        cats.append({"pos": pos, "weights": w, "J": js[i % len(js)], "R": rs[i % len(rs)], "seed": seed})
    return cats


def _twopcf_params(field, R, edges):
    centres = 0.5 * (edges[1:] + edges[:-1])
    return {"Corr_2PCF": {
        "sfc_field": field, "random": "uniform", "window": {"type": "gaussian", "len_args": {"R": float(R)}},
        "binning_window": {"type": "thick_shell", "len_args": {"R": None, "delta_R": float(edges[1] - edges[0])},
                           "mapping": "s_to_R"},
        "sampling": {"s": centres}, "products": ["delta_dd", "xi"]}}


def _threepcf_params(field, radii, lmax, backend="gb300"):
    return {"Corr_3PCF_Multipole": {
        "sfc_field": field, "random": "uniform",
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "grid", "r12": list(radii), "r13": list(radii)},
        "l_min": 0, "l_max": int(lmax), "summation_backend": backend, "products": ["delta_ddd_l", "rrr_l", "zeta_l"]}}


def _project(cat, box, device, workspace=None):
    pos = torch.as_tensor(cat["pos"], device=device)
    return SFCProjection({"SFCProjection": {"particle_pos": pos, "catalog_weight": cat["weights"], "J": cat["J"],
                                            "box_size": box}}, device=device).run(save_result=False)


def run_one_at_a_time(cats, box=1000.0, lmax=6, radii=None, edges=None, device="cuda", backend="gb300"):
    """Each catalogue through the public classes, one after the other."""
    radii = list(np.linspace(10.0, 160.0, 10)) if radii is None else list(radii)
    edges = np.linspace(5.0, 150.0, 21) if edges is None else np.asarray(edges)
    out = []
    for cat in cats:
        f = _project(cat, box, device)
        d2 = Corr_2PCF(_twopcf_params(f, cat["R"], edges), device=device).run(save_result=False)
        d3 = mp.Corr_3PCF_Multipole(_threepcf_params(f, radii, lmax, backend), device=device).run(save_result=False)
        out.append({"xi": np.asarray(d2.xi), "delta_dd": np.asarray(d2.delta_dd), "delta_ddd_l": d3.delta_ddd_l,
                    "zeta_l": d3.zeta_l})
    return out


class BatchPipeline:
    """Batched runner for catalogues of uneven size and J (see the module)."""

    def __init__(self, box=1000.0, lmax=6, radii=None, edges=None, device="cuda", autotune_tiles=True,
                 use_graph=True):
        self.box = float(box)
        self.lmax = int(lmax)
        self.radii = list(np.linspace(10.0, 160.0, 10)) if radii is None else [float(r) for r in radii]
        self.edges = np.linspace(5.0, 150.0, 21) if edges is None else np.asarray(edges, dtype=np.float64)
        self.device = torch.device(device)
        self.autotune_tiles = autotune_tiles
        self.use_graph = use_graph
        self.engines = {}
        self.tiles = {}
        self.deposit_tiles = {}
        self.timing = {}

    def _engine(self, J, phi):
        if J not in self.engines:
            cx, ctas = 0, 0
            if self.autotune_tiles and J >= 4:
                cx, ctas, t = autotune.tune_contract(J, len(self.radii), self.device)
                self.tiles[J] = {"chunk_x": cx, "ctas_per_sm": ctas, "ms": t}
            self.engines[J] = mp.GraphedMultipole(J, self.box, self.radii, self.lmax, phi, self.device, chunk_x=cx,
                                                  ctas_per_sm=ctas, use_graph=self.use_graph)
        return self.engines[J]

    def _tune_deposit(self, J, cat):
        from .phi import sample_scaling_function

        pos = torch.as_tensor(np.asarray(cat["pos"], dtype=np.float64), device=self.device)
        w = torch.as_tensor(np.asarray(cat["weights"], dtype=np.float64), device=self.device)
        phi = torch.as_tensor(sample_scaling_function(), device=self.device)
        tile, ms = autotune.tune_deposit(pos, w, J, self.box, phi)
        self.deposit_tiles[J] = {"tile": "x".join(map(str, tile)), "ms": ms}

    def run(self, cats, group_size=4):
        """Results in input order: dicts with xi, delta_dd, delta_ddd_l, zeta_l."""
        results = [None] * len(cats)
        order = sorted(range(len(cats)), key=lambda i: cats[i]["J"])
        by_j = {}
        for i in order:
            by_j.setdefault(cats[i]["J"], []).append(i)
        pairs = [(a, b) for a in self.radii for b in self.radii]
        for J, idxs in by_j.items():
            if self.autotune_tiles and J not in self.deposit_tiles:
                self._tune_deposit(J, cats[idxs[0]])
            windows = None
            for g0 in range(0, len(idxs), group_size):
                grp = idxs[g0:g0 + group_size]
                fields = [_project(cats[i], self.box, self.device) for i in grp]
                # ---- 2PCF: host set-up by the public task, one pair-product pass for the group
                tasks = [Corr_2PCF(_twopcf_params(f, cats[i]["R"], self.edges), device=self.device)
                         for f, i in zip(fields, grp)]
                specs, dcs = [], []
                for t in tasks:
                    t.prepare_input_fields()
                    d = t.data[1].epsilon_device.to(torch.float32).contiguous()
                    specs.append(rfft_field(d))
                    dcs.append(float(d.double().sum().item()))
                if windows is None:
                    windows = tasks[0]._binning_windows(tasks[0].data[1])
                vals, k0 = pair_products(specs, [(k, k) for k in range(len(grp))], windows, exclude_k0=True)
                L = 1 << J
                for k, (t, i) in enumerate(zip(tasks, grp)):
                    rho = float(t.rand[1])
                    dc = dcs[k] - rho * float(L) ** 3
                    delta_dd = vals[:, k] + dc * dc * k0 / float(L) ** 6
                    factor = float(getattr(t, "_density_physical_scale", 1.0)) ** 2
                    rr = rho * rho
                    if not np.isclose(factor, 1.0):
                        delta_dd = delta_dd * factor
                        rr = rr * factor
                    results[i] = {"delta_dd": delta_dd, "xi": delta_dd / rr}
                del specs
                # ---- 3PCF multipoles: one graph replay per catalogue
                for f, i in zip(fields, grp):
                    t3 = mp.Corr_3PCF_Multipole(_threepcf_params(f, self.radii, self.lmax), device=self.device)
                    t3.prepare_input_fields()
                    ref = t3.reference
                    phi = ref.sfc_info.get("phi_array")
                    eng = self._engine(J, phi)
                    scale = float(getattr(t3, "_density_physical_scale", 1.0)) ** 3
                    delta = t3._eps("delta_ddd_l", 1)
                    ddd = eng.ddd(delta, t3._pairs()) * scale
                    rrr = np.zeros_like(ddd)
                    rrr[:, 0] = t3.rand[1] * t3.rand[2] * t3.rand[3] * scale
                    z, _, cond = mp.mixing_solve(ddd, rrr, self.lmax, device=self.device)
                    results[i].update({"delta_ddd_l": ddd, "rrr_l": rrr, "zeta_l": z, "zeta_condition": cond})
                del fields
        return results
