"""Benchmark of the GB300 field pipeline (one JSON line on rank 0).

Headline workload (one step = one catalogue): spherical-harmonic 3PCF
multipoles.  1,000,000 points Poisson-sampled from a seeded lognormal density
field (P(k) ~ k^-1.5 exp(-(k/0.5 h/Mpc)^2), sigma_G = 1, lognormal(0, 0.3)
weights) and 5,000,000 uniform randoms in a 1000 Mpc/h periodic box are
deposited at J=9 (512^3); delta = D - R (catalogue-normalised); 15 thin
shells over 10-160 Mpc/h on both triangle sides (225 (r12, r13) samples);
l = 0..10; products delta_ddd_l and rrr_l (the random field, full
contraction) and zeta_l (float64 mixing solve).  The step runs through the
public API (Corr_3PCF_Multipole, batched "gb300" backend, tensor-core
contraction engine).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value` = seconds per catalogue, device-timed (CUDA events), inputs already
in HBM.  `e2e` = the same with the catalogues in pinned host memory and the
host->device copies plus the device->host read of zeta_l inside the timed
region.  `plain` = the per-sample reference-form FP32 GPU path (both side
fields rebuilt and a one-pair contraction for every (r12, r13, l, m)), timed
on one full sample (all 66 (l, m) terms) and scaled by the 225 samples and
2 products.  `accuracy_vs_fp64` = the J=8 configuration's unit through the
public API against the committed float64 oracle values (per-l relative
errors).  `roofline` = the batched contraction (mp_contract_tc_kernel), with
the algorithmic FLOPs of the 27-term separable form, 8 * 15 * 15 * 27 * L^3
per (l, m), against the measured bf16 peak; `fields_roofline` = the fields
pass of one (l, m) against HBM.  `traffic` values come from
profiles/ncu_traffic.json (the ncu command and case are recorded there).
`deposit` = the 4M-point J=9 deposit (Mparticles/s, HBM roofline of the
accumulate kernel) with the tile the deposit autotuner picks, the default
tile timed beside it.  `mc3pcf` = Monte Carlo 3PCF on a J=9 lognormal field:
uniform-MC triplets/s on brick-layout fields (C-order fields timed beside
it) and the learned importance-sampling proposal against uniform sampling
(variance per sample, bias, equal-wall-time efficiency).
`c2_window_2pcf` = `field @ W` (gaussian R=10) and the 30x10 (s, mu) ring
2PCF on the 4M-point J=9 field, with their HBM rooflines.  `c4_batched` =
64 uneven catalogues through the batched pipeline against the same public
API one at a time and the plain per-sample path (catalogues/s).
`--impl reference` times the float64 CPU restatement of the reference
(oracle/) at J=9 on the same catalogues (see ReferenceUnits).
Under torchrun each rank runs its own replica catalogue (replicas only: the
path has no exchange step); rank 0 prints the aggregate.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BOX = 1000.0
MP_J = 9
MP_LMAX = 10
MP_NDATA = 1_000_000
MP_NRAND = 5_000_000
MP_RADII = [float(r) for r in np.linspace(10.0, 160.0, 15)]
N_LM = sum(l + 1 for l in range(MP_LMAX + 1))          # 66 (l, m>=0) terms
N_SAMPLES = len(MP_RADII) ** 2                          # 225
METRIC = "zeta_l s/catalogue (J=9, lmax=10, 15x15 shells 10-160 Mpc/h, 1M data + 5M randoms)"
WORKLOAD = ("3PCF multipoles: 1e6 lognormal data + 5e6 uniform randoms deposited at J=9 (512^3), "
            "delta=D-R, 15 thin shells 10-160 Mpc/h on both sides (225 (r12,r13) samples), l=0..10, "
            "products delta_ddd_l + rrr_l (random field) + zeta_l")
DEP_N = 4_000_000
DEP_J = 9
MC_N = 4_000_000          # points of the J=9 lognormal field the MC estimators gather from
MC_CENTRES = 1_000_000    # throughput: centres x rotations = 1e8 triplets
MC_ROT = 100
MC_TRAIN = 10_000_000     # uniform samples the proposal network is trained on
MC_SAMPLES = 100_000_000  # evaluation samples per estimator, split over the test triangles


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def profile_traffic(kernel):
    """DRAM bytes per launch of a kernel from the machine-readable ncu record
    (profiles/ncu_traffic.json: bytes, the captured case, the command and the
    scale to the benchmark's launch), else None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            rec = json.load(f).get(kernel)
    except (OSError, ValueError):
        return None
    if not rec or rec.get("traffic_bytes_per_launch") is None:
        return None
    return float(rec["traffic_bytes_per_launch"]) * float(rec.get("scale", 1))


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def make_catalogues(seed_offset, device):
    """(data pos, data weights, random pos, random weights) as float64 NumPy."""
    from pyhermes_gb300 import synthetic

    dpos, dw = synthetic.lognormal_catalogue(MP_NDATA, box=BOX, seed_field=3 + seed_offset,
                                             seed_poisson=4 + seed_offset, seed_weights=5 + seed_offset,
                                             device=device)
    rng = np.random.default_rng(40 + seed_offset)
    rpos = rng.uniform(0.0, BOX, (MP_NRAND, 3))
    rw = np.ones(MP_NRAND)
    return dpos, dw, rpos, rw


def multipole_task_params(dfield, rfield):
    return {"Corr_3PCF_Multipole": {
        "sfc_field": dfield, "random": rfield,
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "grid", "r12": MP_RADII, "r13": MP_RADII},
        "l_min": 0, "l_max": MP_LMAX, "summation_backend": "gb300", "products": "zeta_l"}}


# ---------------------------------------------------------------------------
# reference arm: the float64 CPU restatement of the reference on the host
# ---------------------------------------------------------------------------
REF_SLABS = 32                      # one step evaluates 1/32 of the grid's x planes
REF_UNITS = ((1, 1), (10, 7))       # (l, m) of the alternating steps
REF_SAMPLE = (MP_RADII[5], MP_RADII[9])


class ReferenceUnits:
    """The reference's per-(sample, l, m) unit (calc_DDD_multipole,
    corr3pcf_multipoles.py:505-555: per side a radial-multipole window and a
    complex FFT convolution, fftn + ifftn; then the 729-term contraction)
    timed at J=9 on the benchmark's own delta field with the oracle's
    float64 restatement on all host threads.  The window and the contraction
    cost the same per grid plane, so a step evaluates both windows on 1/32 of
    the k-space x planes and the contraction on 1/32 of the cells (rotating
    over the slabs); the FFT pair of one convolution is timed once at full
    size.  unit(l) = 32 x slab(l) + 2 x FFT pair, with slab(l) measured at
    l = 1 and l = 10 and linear in l between (the recurrences are O(l))."""

    def __init__(self):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        from scipy.fft import fftn, ifftn

        from pyhermes_gb300.phi import cal_gamma, sample_scaling_function

        self.oracle = oracle
        phi = sample_scaling_function()
        self.L = 1 << MP_J
        self.workers = os.cpu_count() or 1
        dpos, dw, rpos, rw = make_catalogues(0, "cpu")
        t0 = time.perf_counter()
        ed = oracle.deposit(dpos, dw / dw.sum(), phi, MP_J, BOX)
        er = oracle.deposit(rpos, rw / rw.sum(), phi, MP_J, BOX)
        self.t_deposit = time.perf_counter() - t0
        self.delta = ed - er
        del ed, er
        t0 = time.perf_counter()
        spec = fftn(self.delta.astype(np.complex128), workers=self.workers)
        self.field = ifftn(spec, workers=self.workers)
        self.t_fft_pair = time.perf_counter() - t0
        del spec
        self.P = oracle.fourier_power(phi, 1, self.L)
        self.gamma = cal_gamma(phi, 3, 1024)
        self.slab_times = {u: [] for u in REF_UNITS}
        self.k = 0

    def step(self):
        l, m = REF_UNITS[self.k % len(REF_UNITS)]
        slab = (self.k // len(REF_UNITS)) % REF_SLABS
        self.k += 1
        n = self.L // REF_SLABS
        x0, x1 = slab * n, (slab + 1) * n
        o = self.oracle
        t0 = time.perf_counter()
        o.radial_multipole_window_planes(self.L, self.P, REF_SAMPLE[0] * self.L / BOX, l, m, x0, x1)
        o.radial_multipole_window_planes(self.L, self.P, REF_SAMPLE[1] * self.L / BOX, l, -m, x0, x1)
        o.contract_planes(self.delta, self.field, self.field, self.gamma, x0, x1)
        dt = time.perf_counter() - t0
        self.slab_times[(l, m)].append(dt)
        return dt

    def unit_seconds(self, l):
        s1 = statistics.mean(self.slab_times[REF_UNITS[0]])
        s10 = statistics.mean(self.slab_times[REF_UNITS[1]]) if self.slab_times[REF_UNITS[1]] else s1
        slab = s1 + (s10 - s1) * (l - 1) / 9.0
        return REF_SLABS * slab + 2.0 * self.t_fft_pair

    def catalogue_seconds(self):
        return N_SAMPLES * 2 * sum((l + 1) * self.unit_seconds(l) for l in range(MP_LMAX + 1))

    def describe(self):
        return {"value": self.catalogue_seconds(), "unit": "s/catalogue", "cores": self.oracle.num_threads(),
                "kind": "port",
                "sample": (f"J={MP_J} units on the benchmark's delta = D - R (oracle float64 deposit, {self.t_deposit:.1f} s): "
                           f"per step both radial-multipole windows of one (r12, r13) = {REF_SAMPLE} unit on 1/"
                           f"{REF_SLABS} of the k-space x planes plus the 729-term contraction on 1/{REF_SLABS} of "
                           "the cells, alternating (l, m) = (1, 1) and (10, 7); the complex FFT pair of one "
                           f"convolution timed once at full size ({self.t_fft_pair:.2f} s). unit(l) = {REF_SLABS} x "
                           "slab(l) + 2 FFT pairs, slab(l) linear in l between the measured l = 1 and 10; "
                           f"x {N_SAMPLES} samples x sum_l (l+1) (l, m>=0) x 2 products"),
                "unit_s": {"l=1": self.unit_seconds(1), "l=10": self.unit_seconds(10)},
                "slab_s": {f"{l},{m}": statistics.mean(v) for (l, m), v in self.slab_times.items() if v},
                "fft_pair_s": self.t_fft_pair, "slabs": REF_SLABS, "steps_timed": sum(len(v) for v in self.slab_times.values())}


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    ref = ReferenceUnits()
    for _ in range(args.warmup):
        ref.step()
    ref.slab_times = {u: [] for u in REF_UNITS}
    t_steps = []
    for _ in range(max(args.steps, 2)):
        t_steps.append(ref.step())
    per_cat = ref.catalogue_seconds()
    line = {
        "impl": "reference", "metric": METRIC, "value": per_cat, "unit": "s/catalogue",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(t_steps) * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lognormal data + uniform randoms, the GB300 arm's catalogues)",
        "config": {"workload": WORKLOAD, "J": MP_J, "lmax": MP_LMAX},
        "cpu_baseline": ref.describe(),
        "e2e": {"value": per_cat, "unit": "s/catalogue", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def deposit_field(pos_t, w_t, J, phi_t, ws):
    from pyhermes_gb300 import kernels
    from pyhermes_gb300.sfc_field import SFCField

    wsum = float(w_t.sum().item())
    pw = w_t / wsum
    eps, _, _ = kernels.deposit(pos_t, pw, J, BOX, phi_t, workspace=ws)
    L = 1 << J
    f = SFCField(device=pos_t.device)
    f.sfc_info = {"J": J, "L": L, "V": L ** 3, "box_size": BOX, "scale_factor": L / BOX, "phi_resolution": 1024,
                  "wavelet_mode": "db2", "wavelet_level": 10, "phi_support": 3,
                  "phi_array": phi_t.cpu().numpy(), "field_kind": "catalog_field",
                  "weight_normalization": "catalog", "catalog_weight_sum": wsum,
                  "raw_field_weighted_sum": wsum, "field_integral": 1.0, "particle_count": int(pos_t.shape[0])}
    f.format_sfc_params()
    f.epsilon_device = eps
    return f


def deposit_bench(dev, lib, kernels, phi, flush, steps):
    """The 4M-point J=9 deposit: Mparticles/s and the accumulate kernel
    roofline, with the tile the deposit autotuner picks for this catalogue
    (the default 8x16x32 tile timed beside it)."""
    import torch

    from pyhermes_gb300 import _lib, autotune, synthetic

    pos_np, w_np = synthetic.lognormal_catalogue(DEP_N, box=BOX, device=dev)
    pos = torch.as_tensor(pos_np, device=dev)
    pw = torch.as_tensor(w_np / w_np.sum(), device=dev)
    L = 1 << DEP_J
    eps = torch.empty((L, L, L), dtype=torch.float32, device=dev)
    sptr = torch.cuda.current_stream(dev).cuda_stream
    P = ctypes.c_void_p
    stream = torch.cuda.current_stream(dev)

    def measure():
        buf = kernels.DepositWorkspace(dev).get(DEP_N, DEP_J)  # sized for the level's current tile

        def sort():
            _lib.check(lib.hermes_deposit_sort(P(pos.data_ptr()), P(pw.data_ptr()), DEP_N, DEP_J, BOX,
                                               P(phi.data_ptr()), phi.numel(), 1024, P(buf.data_ptr()),
                                               buf.numel(), sptr), "sort")

        def accumulate():
            _lib.check(lib.hermes_deposit_accumulate(DEP_N, DEP_J, BOX, P(phi.data_ptr()), phi.numel(), 1024,
                                                     P(eps.data_ptr()), None, None, P(buf.data_ptr()),
                                                     buf.numel(), sptr), "accumulate")

        for _ in range(3):
            sort()
            accumulate()
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
        torch.cuda.synchronize(dev)
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            sort()
            ev[k][1].record(stream)
            accumulate()
            ev[k][2].record(stream)
        torch.cuda.synchronize(dev)
        step_ms = sum(e[0].elapsed_time(e[2]) for e in ev) / steps
        acc_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / steps
        return step_ms, acc_ms

    autotune.set_deposit_tile(DEP_J, (0, 0, 0))
    default_step, default_acc = measure()
    tile, tile_ms = autotune.tune_deposit(pos, pw, DEP_J, BOX, phi)
    step_ms, acc_ms = measure()
    autotune.set_deposit_tile(DEP_J, (0, 0, 0))
    hbm, _, kind = load_peaks()
    alg = DEP_N * 16 + L ** 3 * 4
    ach = alg / (acc_ms / 1e3) / 1e9
    return {"metric": "deposit Mparticles/s (4M lognormal points, J=9, float32 field)",
            "value": DEP_N / (step_ms / 1e3) / 1e6, "unit": "Mparticles/s",
            "ms_per_step": step_ms, "launches_per_step": 7,
            "tile": "x".join(map(str, tile)), "tile_ms_per_deposit": tile_ms,
            "default_tile": {"tile": "8x16x32", "ms_per_step": default_step, "accumulate_ms": default_acc,
                             "value": DEP_N / (default_step / 1e3) / 1e6},
            "roofline": {"kernel": "dep_accum_kernel", "bound": "hbm", "achieved": ach, "peak": hbm,
                         "peak_kind": kind, "unit": "GB/s", "frac": ach / hbm,
                         "traffic": profile_traffic("dep_accum_kernel"),
                         "algorithmic_bytes": alg, "ms_per_launch": acc_ms}}


def c4_bench(dev, phi_np):
    """64 uneven catalogues (sizes log-uniform in [1e4, 2e6], odd seeds
    uniform, even lognormal, J in {7, 8, 9} and R in {5, 10, 20} Mpc/h
    round-robin), each: deposit, 20-shell 2PCF of the R-smoothed field and
    lmax=6 3PCF multipoles on 10 shells (10-160 Mpc/h).  Catalogues/s of the
    batched pipeline (pyhermes_gb300.batch) against the same public API one
    catalogue at a time, both end to end from host positions and after one
    warm-up catalogue per J (graph capture, tile tuning, cuFFT plans); the
    plain per-sample multipole path is timed on one (r12, r13) sample at
    l <= 1 per J and scaled by samples and (l, m) terms."""
    import torch

    from pyhermes_gb300 import autotune, batch
    from pyhermes_gb300 import multipole as mp

    cats = batch.c4_catalogues(64, box=BOX, device=dev)
    warm = [next(c for c in cats if c["J"] == j) for j in (7, 8, 9)]
    bp = batch.BatchPipeline(box=BOX, device=dev)
    bp.run(warm)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res_b = bp.run(cats)
    torch.cuda.synchronize(dev)
    t_b = time.perf_counter() - t0
    # the one-at-a-time path runs with the default deposit tiles
    for j in (7, 8, 9):
        autotune.set_deposit_tile(j, (0, 0, 0))
    batch.run_one_at_a_time(warm, box=BOX, device=dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res_o = batch.run_one_at_a_time(cats, box=BOX, device=dev)
    torch.cuda.synchronize(dev)
    t_o = time.perf_counter() - t0
    diff = max(float(np.abs(b["zeta_l"] - o["zeta_l"]).max() / np.abs(o["zeta_l"]).max()) for b, o in zip(res_b, res_o))
    diff_xi = max(float(np.abs(b["xi"] - o["xi"]).max() / np.abs(o["xi"]).max()) for b, o in zip(res_b, res_o))
    # plain per-sample multipole path: one sample, l <= 1, per J
    radii = list(np.linspace(10.0, 160.0, 10))
    n_lm = sum(l + 1 for l in range(7))
    plain_unit = {}
    for c in warm:
        f = batch._project(c, BOX, dev)
        t3 = mp.Corr_3PCF_Multipole(batch._threepcf_params(f, radii, 6), device=dev)
        t3.prepare_input_fields()
        d = t3._eps("delta_ddd_l", 1)
        eng = mp.MultipoleEngine(d, d, d, phi_np, c["J"], BOX)
        eng.ddd_plain([(radii[3], radii[6])], 0, 1)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        eng.ddd_plain([(radii[3], radii[6])], 0, 1)
        torch.cuda.synchronize(dev)
        plain_unit[c["J"]] = (time.perf_counter() - t0) / 3.0
    # one-at-a-time time minus its batched-engine multipole share is not separable here; the plain
    # estimate adds the plain multipole cost (100 samples x 28 (l, m)) to the one-at-a-time time
    t_plain = t_o + sum(plain_unit[c["J"]] * len(radii) ** 2 * n_lm for c in cats)
    return {"metric": "catalogues/s (64 uneven catalogues, J in {7,8,9}, 20-shell smoothed 2PCF + lmax=6 "
                      "3PCF multipoles on 10 shells)",
            "value": len(cats) / t_b, "unit": "catalogues/s", "s_batched": t_b,
            "one_at_a_time": {"value": len(cats) / t_o, "s": t_o},
            "plain_estimate": {"value": len(cats) / t_plain, "s": t_plain,
                               "plain_ms_per_sample_lm": {str(k): v * 1e3 for k, v in plain_unit.items()},
                               "sample": "one (r12, r13) sample at l<=1 per J, scaled by 100 samples x 28 (l, m)"},
            "speedup_vs_one_at_a_time": t_o / t_b, "speedup_vs_plain": t_plain / t_b,
            "points_total": int(sum(len(c["weights"]) for c in cats)),
            "max_rel_diff_zeta_batched_vs_one_at_a_time": diff, "max_rel_diff_xi": diff_xi,
            "tiles": {str(k): {"chunk_x": v["chunk_x"], "ctas_per_sm": v["ctas_per_sm"]} for k, v in bp.tiles.items()},
            "deposit_tiles": {str(k): v["tile"] for k, v in bp.deposit_tiles.items()},
            "graph": "one CUDA graph per J: rFFT + 28 x (radial multipole fields + contraction)"}


def c2_bench(dev, phi, steps):
    """4e6 lognormal points at J=9: `field @ W` (gaussian R=10 Mpc/h) and the
    (s, mu) ring 2PCF 30x10 (s 5-150 Mpc/h, mu 0-1, smu_to_RH) through the
    public API, CUDA-event timed with the field in HBM."""
    import torch

    from pyhermes_gb300 import kernels, synthetic
    from pyhermes_gb300.corr2pcf import Corr_2PCF
    from pyhermes_gb300.window import WindowFunc

    pos, w = synthetic.lognormal_catalogue(DEP_N, box=BOX, seed_field=0, seed_poisson=1, seed_weights=2, device=dev)
    f = deposit_field(torch.as_tensor(pos, device=dev), torch.as_tensor(w, device=dev), DEP_J, phi,
                      kernels.DepositWorkspace(dev))
    L = 1 << DEP_J
    stream = torch.cuda.current_stream(dev)
    win = WindowFunc({"type": "gaussian", "len_args": {"R": 10.0}}, f.sfc_info)

    def timed(fn, n):
        for _ in range(2):
            fn()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for a, b in ev:
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize(dev)
        return sum(a.elapsed_time(b) for a, b in ev) / n / 1e3

    t_win = timed(lambda: f @ win, steps)
    s_edges = np.linspace(5.0, 150.0, 31)
    mu_edges = np.linspace(0.0, 1.0, 11)
    task = Corr_2PCF({"Corr_2PCF": {
        "sfc_field": f, "random": "uniform", "binning_window": {"type": "ring"},
        "sampling": {"s": 0.5 * (s_edges[1:] + s_edges[:-1]), "mu": 0.5 * (mu_edges[1:] + mu_edges[:-1])},
        "products": ["delta_dd", "xi"]}}, device=dev)
    t_2pcf = timed(lambda: task.run(save_result=False), steps)
    hbm, _, kind = load_peaks()
    real_b, half_b = L ** 3 * 4, L * L * (L // 2 + 1) * 8
    win_bytes = 2 * (real_b + half_b) + 2 * half_b  # rFFT r+w, irFFT r+w, window pass r+w
    tp_bytes = real_b + 2 * half_b                  # rFFT of the field + one read of the half spectrum
    return {"metric": "field @ gaussian(R=10) and 30x10 (s, mu) ring 2PCF, 4e6 lognormal points, J=9",
            "window_ms": t_win * 1e3, "twopcf_ms": t_2pcf * 1e3, "twopcf_bins": 300,
            "window_roofline": {"bound": "hbm", "achieved": win_bytes / t_win / 1e9, "peak": hbm, "peak_kind": kind,
                                "unit": "GB/s", "frac": win_bytes / t_win / 1e9 / hbm,
                                "algorithmic_bytes": win_bytes,
                                "note": "cuFFT R2C + on-the-fly window multiply + cuFFT C2R"},
            "twopcf_roofline": {"bound": "hbm", "achieved": tp_bytes / t_2pcf / 1e9, "peak": hbm,
                                "peak_kind": kind, "unit": "GB/s", "frac": tp_bytes / t_2pcf / 1e9 / hbm,
                                "algorithmic_bytes": tp_bytes,
                                "traffic": profile_traffic("pair_products_cylz_kernel"),
                                "note": "one forward rFFT and one pass over the half spectrum for all 300 bins "
                                        "(separable ring windows, column kernel); issue-bound"}}


def mc_bench(dev, phi_np, steps):
    """Monte Carlo 3PCF on a J=9 lognormal field (4e6 points): uniform-MC
    triplet throughput of hermes_mc_triplets (1e6 centres x 100 rotations),
    and the learned importance-sampling proposal (trained on 1e7 uniform
    samples over r12, r13 in [20, 120] Mpc/h, mu in [-1, 1]) against uniform
    sampling on three test triangles in the reference estimator's form
    (centres x 100 rotations, hermes_mc_triplets with centre weights; the
    learned centres are drawn from the proposal over a fresh uniform pool of
    16x candidates per replicate; the proposal sees the centre density and
    the shell-averaged densities at r12 and r13), 64 independent replicates
    of ~5e5 triplets per triangle and estimator: estimator variance from the
    replicate spread, bias in units of the combined standard error, and
    variance x time at equal wall time (the learned time includes the
    proposal on the candidate pools)."""
    import torch

    from pyhermes_gb300 import kernels, mc3pcf, synthetic

    L = 1 << DEP_J
    sc = L / BOX
    pos, w = synthetic.lognormal_catalogue(MC_N, box=BOX, seed_field=0, seed_poisson=1, seed_weights=2, device=dev)
    phi = torch.as_tensor(phi_np, device=dev)
    eps, _, _ = kernels.deposit(torch.as_tensor(pos, device=dev), torch.as_tensor(w / w.sum(), device=dev), DEP_J,
                                BOX, phi)
    rho = 1.0 / L ** 3
    lp = mc3pcf.LearnedProposal(eps, eps, eps, DEP_J, phi_np, rho, device=dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(7)
    cen = torch.as_tensor(rng.uniform(0.0, L, (MC_CENTRES, 3)), device=dev)
    off = mc3pcf.rotation_offsets(50.0 * sc, 80.0 * sc, 0.5, MC_ROT, rng=np.random.RandomState(8))
    def time_triplets(bricks):
        for _ in range(2):
            mc3pcf.triplet_sum(lp.e1, lp.e2, lp.e3, DEP_J, cen, off, lp.phi_t, bricks=bricks)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for a, b in ev:
            a.record(stream)
            mc3pcf.triplet_sum(lp.e1, lp.e2, lp.e3, DEP_J, cen, off, lp.phi_t, bricks=bricks)
            b.record(stream)
        torch.cuda.synchronize(dev)
        return sum(a.elapsed_time(b) for a, b in ev) / len(ev) / 1e3

    t_c_order = time_triplets(False)  # fields in C order, as the reference stores them
    t_tr = time_triplets(True)        # brick-layout copies (the default path)
    ntr = MC_CENTRES * MC_ROT
    hbm, _, kind = load_peaks()
    ach = ntr * 324 / t_tr / 1e9

    grid_r = [20.0, 53.3, 86.7, 120.0]
    configs = [(r1 * sc, r2 * sc, mu) for r1 in grid_r for r2 in grid_r if r2 >= r1 for mu in (-0.75, -0.25, 0.25, 0.75)]
    n_rot_train = 32
    n_cen_train = MC_TRAIN // (len(configs) * n_rot_train)
    t0 = time.perf_counter()
    losses = lp.train(configs, n_centers=n_cen_train, n_rot_train=n_rot_train, epochs=3, seed=1)
    torch.cuda.synchronize(dev)
    t_train = time.perf_counter() - t0
    tests = [(30.0, 60.0, 0.8), (60.0, 90.0, -0.3), (100.0, 120.0, 0.0)]
    n_rot = 100
    pool_factor = 16
    replicates = 64
    n_cen = MC_SAMPLES // (len(tests) * n_rot * replicates)  # centres per replicate
    rows = []
    for k, (r1, r2, mu) in enumerate(tests):
        args = (r1 * sc, r2 * sc, mu, n_cen, n_rot)
        lp.centre_estimate(*args, seed=1, replicates=2, pool_factor=pool_factor)  # warm-up
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        mu_u, se_u = lp.centre_estimate(*args, seed=100 + k, uniform=True, replicates=replicates)
        torch.cuda.synchronize(dev)
        t_u = time.perf_counter() - t0
        t0 = time.perf_counter()
        # includes the proposal on fresh candidate pools
        mu_l, se_l = lp.centre_estimate(*args, seed=200 + k, pool_factor=pool_factor, replicates=replicates)
        torch.cuda.synchronize(dev)
        t_l = time.perf_counter() - t0
        se = float(np.sqrt(se_u ** 2 + se_l ** 2))
        rows.append({"r12": r1, "r13": r2, "mu": mu, "triplets": replicates * n_cen * n_rot,
                     "centres_per_replicate": n_cen,
                     "rotations": n_rot, "mean_uniform": mu_u, "mean_learned": mu_l, "stderr_uniform": se_u,
                     "stderr_learned": se_l, "variance_ratio_equal_samples": (se_u / se_l) ** 2,
                     "bias_sigma": (mu_l - mu_u) / se, "s_uniform": t_u, "s_learned": t_l,
                     "efficiency_equal_wall_time": (se_u ** 2 * t_u) / (se_l ** 2 * t_l)})
    return {"metric": "uniform-MC triplet samples/s (J=9 lognormal field from 4e6 points)",
            "value": ntr / t_tr, "unit": "triplets/s", "ms_per_launch": t_tr * 1e3,
            "c_order_fields": {"value": ntr / t_c_order, "ms_per_launch": t_c_order * 1e3},
            "sample": f"{MC_CENTRES} centres x {MC_ROT} rotations, r12=50, r13=80 Mpc/h, mu=0.5",
            "roofline": {"kernel": "mc_triplet_kernel<bricks>", "bound": "hbm", "achieved": ach, "peak": hbm,
                         "peak_kind": kind, "unit": "GB/s", "frac": ach / hbm,
                         "algorithmic_bytes_per_triplet": 324,
                         "traffic": profile_traffic("mc_triplet_kernel"),
                         "note": "3 x 27 float32 gathers per triplet over Morton-ordered centres, fields in "
                                 "2x2x2 bricks (one 32-byte sector each)"},
            "learned_proposal": {"train_samples": len(configs) * n_cen_train * n_rot_train,
                                 "train_s": t_train, "loss_first_last": [losses[0], losses[-1]],
                                 "pool_factor": pool_factor, "replicates": replicates, "tests": rows}}


def run_case(args):
    """Single-part workloads for profiling (`--case step|contract|fields|
    deposit|mc|c2|c4`): one JSON line with CUDA-event times; not the headline
    line (`step` is the headline step alone, for launch lists).
    `fields` is one radial multipole fields call (l=4, m=2, the 15 headline
    radii) on the deposited lognormal field at level --J."""
    import torch

    from pyhermes_gb300 import _lib, kernels, synthetic
    from pyhermes_gb300 import multipole as mp
    from pyhermes_gb300.phi import cal_gamma, sample_scaling_function
    from pyhermes_gb300.window import phi_power_device, rfft_field

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    phi_np = sample_scaling_function()
    phi = torch.as_tensor(phi_np, device=dev)
    stream = torch.cuda.current_stream(dev)
    if args.case == "c4":
        print(json.dumps({"case": "c4", **c4_bench(dev, phi_np)}))
        return 0
    if args.case == "c2":
        print(json.dumps({"case": "c2", **c2_bench(dev, phi, args.steps)}))
        return 0
    if args.case == "mc":
        print(json.dumps({"case": "mc", **mc_bench(dev, phi_np, args.steps)}))
        return 0
    if args.case == "step":
        # the headline step alone (deposits, fields, contractions, mixing solve), W + K times
        dpos_np, dw_np, rpos_np, rw_np = make_catalogues(0, "cpu")
        t = [torch.as_tensor(a, device=dev) for a in (dpos_np, dw_np, rpos_np, rw_np)]
        wsd, wsr = kernels.DepositWorkspace(dev), kernels.DepositWorkspace(dev)

        def step():
            task = mp.Corr_3PCF_Multipole(multipole_task_params(deposit_field(t[0], t[1], MP_J, phi, wsd),
                                                                deposit_field(t[2], t[3], MP_J, phi, wsr)),
                                          device=dev)
            return task.run(save_result=False)

        for _ in range(args.warmup):
            step()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in ev:
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize(dev)
        print(json.dumps({"case": "step", "s_per_catalogue": sum(a.elapsed_time(b) for a, b in ev) / len(ev) / 1e3,
                          "steps": args.steps, "warmup": args.warmup}))
        return 0
    if args.case == "deposit":
        flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
        out = deposit_bench(dev, _lib.load(), kernels, phi, flush, args.steps)
        print(json.dumps({"case": "deposit", **out}))
        return 0
    J = args.J
    L = 1 << J
    pos, w = synthetic.lognormal_catalogue(MP_NDATA, box=BOX, ng=min(L, 256), device=dev)
    pw = torch.as_tensor(w / w.sum(), device=dev)
    eps, _, _ = kernels.deposit(torch.as_tensor(pos, device=dev), pw, J, BOX, phi)
    eps = (eps - eps.double().mean().float()).contiguous()
    P = phi_power_device(phi_np, L, 1, 1024, dev)
    gam = cal_gamma(phi_np, 3, 1024)
    grid = [r * L / BOX for r in MP_RADII]
    if args.case == "fields":
        spec = rfft_field(eps)
        res = {}
        for bm in (True, False):
            out = mp._fields_out(J, len(grid), bm, dev)
            wsf = mp._workspace(mp.fields_ws_bytes(J, len(grid), bm), dev)
            for _ in range(max(args.warmup, 1)):
                mp.multipole_fields(spec, J, 4, 2, grid, P, out=out, ws=wsf, bin_major=bm)
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
            for a, b in ev:
                a.record(stream)
                mp.multipole_fields(spec, J, 4, 2, grid, P, out=out, ws=wsf, bin_major=bm)
                b.record(stream)
            torch.cuda.synchronize(dev)
            res["bin_major" if bm else "interleaved"] = sum(a.elapsed_time(b) for a, b in ev) / len(ev)
            del out
        print(json.dumps({"case": "fields", "J": J, "bins": len(grid), "l": 4, "m": 2, "ms_per_call": res,
                          "prepass_bytes_written": len(grid) * L ** 3 * 8}))
        return 0
    rfield = rfft_field(eps)
    gc = (ctypes.c_double * 9)(*np.asarray(gam, dtype=np.float64).ravel())
    dout = torch.zeros((16, 16, 2), dtype=torch.float64, device=dev)
    res = {}
    variants = {"tensor_bm": ("tensor", True), "tensor": ("tensor", False), "simt": ("simt", False)}
    chosen = [v for v in args.variants.split(",") if v] if args.variants else ["tensor_bm", "simt"]
    for name in chosen:
        engine, bm = variants[name]
        f = mp.multipole_fields(rfield, J, 2, 1, grid, P, bin_major=bm)
        for _ in range(max(args.warmup, 1)):
            mp.multipole_contract_async(eps, f, len(grid), gc, J, dout, conj_sign=-1, engine=engine, bin_major=bm)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in ev:
            a.record(stream)
            mp.multipole_contract_async(eps, f, len(grid), gc, J, dout, conj_sign=-1, engine=engine, bin_major=bm)
            b.record(stream)
        torch.cuda.synchronize(dev)
        S = dout[:len(grid), :len(grid)].cpu().numpy()
        res[name] = {"ms_per_launch": sum(a.elapsed_time(b) for a, b in ev) / len(ev), "S": S[..., 0] + 1j * S[..., 1]}
        del f
    del rfield
    diff = {k: float(np.abs(v["S"] - res["simt"]["S"]).max() / np.abs(res["simt"]["S"]).max())
            for k, v in res.items() if k != "simt" and "simt" in res}
    print(json.dumps({"case": "contract", "J": J, "bins": len(grid), "l": 2, "m": 1,
                      "ms_per_launch": {k: v["ms_per_launch"] for k, v in res.items()},
                      "max_rel_diff_vs_simt": diff, "status": mp.contract_status(J, device=dev),
                      "algorithmic_flops": 8.0 * len(grid) ** 2 * 27 * L ** 3}))
    return 0


def accuracy_vs_fp64(dev, engine="tensor"):
    """The 3PCF-multipole unit of the J=8 configuration (1,000,000 lognormal
    points + 5,000,000 uniform randoms, delta = D - R, one (r12, r13) = (50,
    90) Mpc/h sample, l = 0..10) through the public API (GPU deposit,
    fields, contraction, mixing solve) against the float64 oracle's values
    committed in tests/golden/c3_unit_J8.npz: per-l relative errors."""
    path = os.path.join(ROOT, "tests", "golden", "c3_unit_J8.npz")
    if not os.path.exists(path):
        return None
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_multipole_fixtures as fx

    from pyhermes_gb300 import multipole as mp
    from pyhermes_gb300.projection import SFCProjection

    g = np.load(path)
    seeds = dict(zip(("field", "poisson", "jitter", "weights", "random"), (int(v) for v in g["seeds"])))
    pos, w, rpos = fx.unit_positions(fx.unit_cells_decode(int(g["cells_first"]), g["cells_diff"]), seeds, int(g["ng"]),
                                     int(g["n_rand"]))
    J = int(g["J"])
    d = SFCProjection({"SFCProjection": {"particle_pos": pos, "catalog_weight": w, "J": J, "box_size": BOX}},
                      device=dev).run(save_result=False)
    r = SFCProjection({"SFCProjection": {"particle_pos": rpos, "J": J, "box_size": BOX}}, device=dev).run(
        save_result=False)
    res = mp.Corr_3PCF_Multipole({"Corr_3PCF_Multipole": {
        "sfc_field": d, "random": r,
        "binning_window12": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r12"}},
        "binning_window13": {"type": "shell", "len_args": {}, "other_args": {}, "mapping": {"R": "r13"}},
        "sampling": {"mode": "paired", "r12": [float(g["r12"])], "r13": [float(g["r13"])]},
        "l_min": 0, "l_max": int(g["lmax"]), "products": "zeta_l", "contraction_engine": engine}},
        device=dev).run(save_result=False)
    out = {}
    for k in ("zeta_l", "delta_ddd_l", "rrr_l"):
        got = np.asarray(getattr(res, k))
        e = np.abs(got - g[k]) / np.abs(g[k])
        es = np.abs(got - g[k]) / np.abs(g[k]).max()
        out[k] = {"max_per_value": float(e.max()), "max_over_sample_max": float(es.max()),
                  "per_l": [float(x) for x in e.ravel()]}
    return {"engine": engine, "case": "J=8, 1e6 lognormal + 5e6 uniform randoms, (r12, r13) = (50, 90) Mpc/h, l<=10",
            "max_rel_err_zeta_l": out["zeta_l"]["max_per_value"], "per_product": out}


def run_gb300(args, ws, rank, local):
    import torch

    from pyhermes_gb300 import _lib, kernels
    from pyhermes_gb300 import multipole as mp
    from pyhermes_gb300.phi import sample_scaling_function

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    lib = _lib.load()
    phi_np = sample_scaling_function()
    phi = torch.as_tensor(phi_np, device=dev)
    dpos_np, dw_np, rpos_np, rw_np = make_catalogues(rank, "cpu")
    dpos, dw = torch.as_tensor(dpos_np, device=dev), torch.as_tensor(dw_np, device=dev)
    rpos, rw = torch.as_tensor(rpos_np, device=dev), torch.as_tensor(rw_np, device=dev)
    wsd, wsr = kernels.DepositWorkspace(dev), kernels.DepositWorkspace(dev)
    stream = torch.cuda.current_stream(dev)

    def step(dp, dwt, rp, rwt):
        dfield = deposit_field(dp, dwt, MP_J, phi, wsd)
        rfield = deposit_field(rp, rwt, MP_J, phi, wsr)
        task = mp.Corr_3PCF_Multipole(multipole_task_params(dfield, rfield), device=dev)
        return task.run(save_result=False)

    for _ in range(max(args.warmup, 3) if args.warmup > 0 else 0):
        res = step(dpos, dw, rpos, rw)
    torch.cuda.synchronize(dev)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize(dev)
    for k in range(args.steps):
        ev[k][0].record(stream)
        res = step(dpos, dw, rpos, rw)
        ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    clk = clocks.stop()
    t_total = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    if ws > 1:
        from pyhermes_gb300.replicas import max_over_ranks

        t_total = max_over_ranks(t_total, device=dev)
    # whole-job: catalogues per second over all ranks -> seconds per catalogue
    value = t_total / (args.steps * ws)
    zeta = np.asarray(res.zeta_l)

    # our kernels per step: 2 deposits x 7; per product, per single (l, m) term 8 (fields: power,
    # j_l table, interior and edge prepass, the y and x FFT passes after cuFFT's z lines; contract:
    # tensor-core contraction, reduce) and per degree pair 9 (a second j_l table); the mixing solve
    n_pairs = len(mp.degree_pairs([(l, m) for l in range(MP_LMAX + 1) for m in range(l + 1)]))
    kernel_launches = args.steps * (14 + 2 * ((N_LM - 2 * n_pairs) * 8 + n_pairs * 9) + 1)

    # end to end: catalogues in pinned host memory, copies inside the timed region
    h = [torch.as_tensor(a).pin_memory() for a in (dpos_np, dw_np, rpos_np, rw_np)]
    d = [torch.empty_like(x, device=dev) for x in h]
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    for k in range(args.steps):
        e2e_ev[k][0].record(stream)
        for src, dst in zip(h, d):
            dst.copy_(src, non_blocking=True)
        r2 = step(*d)
        np.asarray(r2.zeta_l)  # zeta_l read back to the host (done inside run())
        e2e_ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    e2e_value = sum(a.elapsed_time(b) for a, b in e2e_ev) / 1e3 / (args.steps * ws)

    # dominant kernel: the batched contraction of one (l, m) over 15x15 radii, the tensor engine on
    # the bin-major fields the headline path uses and the FP32 engine on the interleaved layout; the
    # fields pass of the same (l, m) in both layouts
    dfield = deposit_field(dpos, dw, MP_J, phi, wsd)
    rfield = deposit_field(rpos, rw, MP_J, phi, wsr)
    delta = (dfield.epsilon_device.double() - rfield.epsilon_device.double()).float()
    del dfield, rfield
    eng = mp.MultipoleEngine(delta, delta, delta, phi_np, MP_J, BOX)
    L = 1 << MP_J
    grid = [r * L / BOX for r in MP_RADII]
    gc = (ctypes.c_double * 9)(*np.asarray(eng.gamma, dtype=np.float64).ravel())
    dout = torch.zeros((16, 16, 2), dtype=torch.float64, device=dev)
    t_con, t_fld = {}, {}
    for engine, bm in (("tensor", True), ("simt", False)):
        f2 = mp.multipole_fields(eng.spec2, MP_J, 4, 2, grid, eng.P, bin_major=bm)
        for _ in range(2):
            mp.multipole_contract_async(eng.eps1, f2, 15, gc, MP_J, dout, conj_sign=1, engine=engine, bin_major=bm)
        cev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
        for a, b in cev:
            a.record(stream)
            mp.multipole_contract_async(eng.eps1, f2, 15, gc, MP_J, dout, conj_sign=1, engine=engine, bin_major=bm)
            b.record(stream)
        torch.cuda.synchronize(dev)
        t_con[engine] = sum(a.elapsed_time(b) for a, b in cev) / len(cev) / 1e3
        fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
        for a, b in fev:
            a.record(stream)
            mp.multipole_fields(eng.spec2, MP_J, 4, 2, grid, eng.P, out=f2, bin_major=bm)
            b.record(stream)
        torch.cuda.synchronize(dev)
        t_fld["bin_major" if bm else "interleaved"] = sum(a.elapsed_time(b) for a, b in fev) / len(fev) / 1e3
        del f2
    hbm, bf16, kind = load_peaks()
    flops = 8.0 * 15 * 15 * 27 * L ** 3
    stencil_flops = 81 * 2 * 2 * 16 * L ** 3 * (128 + 4) / 128
    achieved = flops / t_con["tensor"] / 1e12
    fld_bytes = L * L * (L // 2 + 1) * 8 + L ** 3 * 15 * 8

    # plain per-sample reference-form path: one full (r12, r13) sample over every (l, m), l <= 10
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    plain = eng.ddd_plain([REF_SAMPLE], 0, MP_LMAX)
    torch.cuda.synchronize(dev)
    t_plain_sample = time.perf_counter() - t0
    plain_per_cat = t_plain_sample * N_SAMPLES * 2
    batched = eng.ddd([REF_SAMPLE], 0, MP_LMAX)
    plain_diff = np.abs(batched - plain) / np.abs(plain)
    del eng, delta

    acc = accuracy_vs_fp64(dev)

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    dep = deposit_bench(dev, lib, kernels, phi, flush, max(args.steps, 5))
    mc = mc_bench(dev, phi_np, max(args.steps, 3))
    c2 = c2_bench(dev, phi, max(args.steps, 3))
    c4 = c4_bench(dev, phi_np)

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return 0
    ref = ReferenceUnits()
    for _ in range(2):
        ref.step()
    cpu = ref.describe()
    line = {
        "metric": METRIC, "value": value, "unit": "s/catalogue", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 fields and stencil, bf16x3 tensor-core bin product, f64 reductions and mixing solve",
        "data": "synthetic (seeded lognormal data + uniform randoms; the reference's Quijote catalogue is absent)",
        "config": {"workload": WORKLOAD, "J": MP_J, "lmax": MP_LMAX, "radii": len(MP_RADII),
                   "samples": N_SAMPLES, "n_data": MP_NDATA, "n_random": MP_NRAND,
                   "l2": "per-(l,m) working set (16 GB fields) far above L2",
                   "parallelism": f"replicas x{ws}"},
        "accuracy_vs_fp64": acc,
        "max_rel_err_vs_fp64": None if acc is None else acc["max_rel_err_zeta_l"],
        "plain": {"value": plain_per_cat, "unit": "s/catalogue", "speedup_mixed_batched_vs_plain": plain_per_cat / value,
                  "sample_s": t_plain_sample,
                  "sample": (f"one full (r12, r13) = {REF_SAMPLE} sample, all 66 (l, m>=0) terms l<=10: per-sample "
                             "single-radius fields and the reference-form FP32 contraction, x225 samples x2 products"),
                  "max_rel_diff_batched_vs_plain_per_l": float(plain_diff.max())},
        "roofline": {"kernel": "mp_contract_tc_kernel (+ mp_reduce_kernel)", "bound": "tensor",
                     "achieved": achieved, "peak": bf16, "peak_kind": kind, "unit": "TFLOP/s",
                     "frac": achieved / bf16, "traffic": profile_traffic("mp_contract_tc_kernel"),
                     "executes_on": ("stencil on FP32 paired-FMA pipes; bin x bin product on tcgen05 "
                                     "(BF16x3 operands, FP32 accumulate in TMEM)"),
                     "algorithmic_flops": flops, "ms_per_launch": t_con["tensor"] * 1e3,
                     "ms_per_launch_simt_engine": t_con["simt"] * 1e3,
                     # what bounds the kernel: the FP32 stencil on the CUDA cores (81 paired
                     # complex x real FMAs per cell, bin lane and x-plane; 16 bin lanes; the
                     # 4-plane halo of each 128-plane x-chunk) against the nominal FP32 peak
                     # (152 SMs x 128 lanes x 2 FLOP x 2.07 GHz)
                     "stencil_fp32": {"flops": stencil_flops, "achieved_tflops": stencil_flops / t_con["tensor"] / 1e12,
                                      "nominal_peak_tflops": 80.6,
                                      "frac": stencil_flops / t_con["tensor"] / 1e12 / 80.6}},
        "fields_roofline": {"kernels": "mp_jl_table + mp_prepass_quad/edge + inverse FFT of 15 fields (cuFFT 1-D z "
                                       "lines, fft512_cols_kernel over y and x; bin-major output, read as is by the "
                                       "tensor-core contraction)",
                            "bound": "hbm", "ms_per_lm": t_fld["bin_major"] * 1e3, "algorithmic_bytes": fld_bytes,
                            "achieved": fld_bytes / t_fld["bin_major"] / 1e9, "peak": hbm, "peak_kind": kind,
                            "unit": "GB/s", "frac": fld_bytes / t_fld["bin_major"] / 1e9 / hbm,
                            "ms_per_lm_interleaved": t_fld["interleaved"] * 1e3,
                            "note": "minimum bytes: one read of the half spectrum + one write of the 15 fields; "
                                    "the interleaved layout (FP32 engine) adds the mp_interleave pass"},
        "deposit": dep,
        "mc3pcf": mc,
        "c2_window_2pcf": c2,
        "c4_batched": c4,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "s/catalogue",
                "h2d_bytes_per_step": int(sum(x.numel() * x.element_size() for x in h)),
                "d2h_bytes_per_step": int(zeta.size * 8)},
        "gpu_launches": kernel_launches,
        "zeta_l_shape": list(zeta.shape),
        "clocks": clk,
    }
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--case", default="headline", choices=["headline", "step", "contract", "fields", "deposit", "mc", "c2",
                                                           "c4"],
                    help="headline = the benchmark line; contract/fields/deposit/mc/c2/c4 = one part, for profiling")
    ap.add_argument("--J", type=int, default=7, help="grid level of --case contract and --case fields")
    ap.add_argument("--variants", default="", help="--case contract: comma list of tensor_bm, tensor, simt")
    args = ap.parse_args()
    if args.case != "headline":
        return run_case(args)
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_gb300(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
