"""Benchmark of the GB300 field pipeline (one JSON line on rank 0).

Workload (default): the clustered-field deposit configuration — 4,000,000
points Poisson-sampled from a seeded lognormal density field
(P(k) ~ k^-1.5 exp(-(k/0.5)^2), sigma_G = 1) in a 1000 Mpc/h periodic box,
lognormal(0, 0.3) weights, projected at J=9 (512^3 float32 coefficients).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value` is device-timed whole-job throughput with inputs resident in HBM;
`e2e` is the same metric through the C ABI with host (pinned) inputs, the
host->device copy and the device->host read of the field inside the timed
region.  `--impl reference` times the float64 CPU restatement of the
reference deposit (oracle/, sequential like the reference loop) on the
host.  Under torchrun each rank deposits its own replica catalogue (replicas
only: the path has no exchange step); rank 0 prints.
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

N_PARTICLES = 4_000_000
J = 9
BOX = 1000.0
METRIC = "deposit Mparticles/s (4M lognormal points, J=9, float32 coefficients)"
WORKLOAD = "clustered lognormal catalogue deposit: 4e6 points, J=9 (512^3), box 1000 Mpc/h"


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_catalogue(seed_offset, device):
    from pyhermes_gb300 import synthetic

    pos, w = synthetic.lognormal_catalogue(N_PARTICLES, box=BOX, seed_field=0 + seed_offset,
                                           seed_poisson=1 + seed_offset, seed_weights=2 + seed_offset,
                                           device=device)
    pw = w / w.sum()
    return pos, pw


def cpu_deposit_rate(pos, pw, phi, n_sample):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    t0 = time.perf_counter()
    oracle.deposit(pos[:n_sample], pw[:n_sample], phi, J, BOX)
    dt = time.perf_counter() - t0
    return n_sample / dt / 1e6, dt


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    from pyhermes_gb300.phi import sample_scaling_function

    device = "cuda" if _cuda_ok() else "cpu"
    pos, pw = make_catalogue(0, device if device == "cuda" else "cpu")
    phi = sample_scaling_function()
    for _ in range(args.warmup):
        cpu_deposit_rate(pos, pw, phi, N_PARTICLES // 4)
    rates, total = [], 0.0
    for _ in range(args.steps):
        r, dt = cpu_deposit_rate(pos, pw, phi, N_PARTICLES)
        rates.append(r)
        total += dt
    value = N_PARTICLES * args.steps / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mparticles/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded lognormal catalogue)",
        "config": {"workload": WORKLOAD, "n_particles": N_PARTICLES, "J": J},
        "cpu_baseline": {"value": value, "unit": "Mparticles/s", "cores": 1, "kind": "port",
                         "sample": f"full {N_PARTICLES} particle catalogue per step, sequential float64 "
                                   "restatement of the reference deposit loop (oracle/hermes_oracle.c)"},
        "e2e": {"value": value, "unit": "Mparticles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _cuda_ok():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def run_gb300(args, ws, rank, local):
    import torch

    from pyhermes_gb300 import _lib, kernels
    from pyhermes_gb300.phi import sample_scaling_function

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    lib = _lib.load()
    pos_np, pw_np = make_catalogue(rank, dev)
    phi_np = sample_scaling_function()
    pos = torch.as_tensor(pos_np, device=dev)
    pw = torch.as_tensor(pw_np, device=dev)
    phi = torch.as_tensor(phi_np, device=dev)
    L = 1 << J
    eps = torch.empty((L, L, L), dtype=torch.float32, device=dev)
    wsp = kernels.DepositWorkspace(dev)
    buf = wsp.get(N_PARTICLES, J)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    P = ctypes.c_void_p

    def sort():
        _lib.check(lib.hermes_deposit_sort(P(pos.data_ptr()), P(pw.data_ptr()), N_PARTICLES, J, BOX,
                                           P(phi.data_ptr()), phi.numel(), 1024, P(buf.data_ptr()),
                                           buf.numel(), sptr), "sort")

    def accumulate():
        _lib.check(lib.hermes_deposit_accumulate(N_PARTICLES, J, BOX, P(phi.data_ptr()), phi.numel(), 1024,
                                                 P(eps.data_ptr()), None, None, P(buf.data_ptr()),
                                                 buf.numel(), sptr), "accumulate")

    for _ in range(max(args.warmup, 3)):
        sort()
        accumulate()
    torch.cuda.synchronize(dev)
    kernels_per_step = 7  # max, bin, 3 scan phases, scatter, accumulate

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize(dev)
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        sort()
        ev[k][1].record(stream)
        accumulate()
        ev[k][2].record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    clk = clocks.stop()
    step_ms = [e[0].elapsed_time(e[2]) for e in ev]
    acc_ms = [e[1].elapsed_time(e[2]) for e in ev]
    t_total = sum(step_ms) / 1e3
    if ws > 1:
        import torch.distributed as dist

        t = torch.tensor([t_total], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_total = float(t.item())
    value = N_PARTICLES * ws * args.steps / t_total / 1e6

    # end to end through the C ABI: pinned host buffers, H2D + deposit + D2H of the field
    pos_h = torch.as_tensor(pos_np).pin_memory()
    pw_h = torch.as_tensor(pw_np).pin_memory()
    eps_h = torch.empty((L, L, L), dtype=torch.float32).pin_memory()
    pos_d = torch.empty_like(pos)
    pw_d = torch.empty_like(pw)
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    for k in range(args.steps + 1):
        flush.zero_()
        if k > 0:
            e2e_ev[k - 1][0].record(stream)
        pos_d.copy_(pos_h, non_blocking=True)
        pw_d.copy_(pw_h, non_blocking=True)
        _lib.check(lib.hermes_deposit(P(pos_d.data_ptr()), P(pw_d.data_ptr()), N_PARTICLES, J, BOX,
                                      P(phi.data_ptr()), phi.numel(), 1024, P(eps.data_ptr()), None, None,
                                      P(buf.data_ptr()), buf.numel(), sptr), "deposit")
        eps_h.copy_(eps, non_blocking=True)
        if k > 0:
            e2e_ev[k - 1][1].record(stream)
    torch.cuda.synchronize(dev)
    e2e_s = sum(a.elapsed_time(b) for a, b in e2e_ev) / 1e3
    e2e_value = N_PARTICLES * ws * args.steps / e2e_s / 1e6

    peak, peak_kind = load_peaks()
    alg_bytes = N_PARTICLES * 16 + L ** 3 * 4
    acc_mean = sum(acc_ms) / len(acc_ms) / 1e3
    achieved = alg_bytes / acc_mean / 1e9
    pass_bytes = N_PARTICLES * (24 + 8) + L ** 3 * 4
    pass_gbs = pass_bytes / (t_total / args.steps) / 1e9

    if rank != 0:
        return 0
    cpu_rate, cpu_dt = cpu_deposit_rate(pos_np, pw_np, phi_np, 1_000_000)
    line = {
        "metric": METRIC, "value": value, "unit": "Mparticles/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded lognormal catalogue; the reference's Quijote catalogue is not available)",
        "config": {"workload": WORKLOAD, "n_particles": N_PARTICLES, "J": J, "box": BOX,
                   "l2": "flushed (256 MiB write) before every timed step; field 512 MiB > L2",
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"kernel": "dep_accum_kernel", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None,
                     "algorithmic_bytes": alg_bytes, "ms_per_launch": acc_mean * 1e3},
        "deposit_pass": {"GB/s": pass_gbs, "frac": pass_gbs / peak,
                         "algorithmic_bytes": pass_bytes,
                         "note": "all 7 kernels; float64 xyz+w in, float32 field out"},
        "cpu_baseline": {"value": cpu_rate, "unit": "Mparticles/s", "cores": 1, "kind": "port",
                         "sample": "first 1,000,000 particles of the catalogue, sequential float64 "
                                   f"restatement of the reference loop ({cpu_dt:.2f} s)"},
        "e2e": {"value": e2e_value, "unit": "Mparticles/s",
                "h2d_bytes_per_step": N_PARTICLES * 32, "d2h_bytes_per_step": L ** 3 * 4},
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_gb300(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
