"""Acquisition throughput benchmark (cells/s; one cell = PRN x Doppler x code phase).

Default workload: batched multi-constellation acquisition of one 40 ms
capture of int16 I/Q at 50 MHz (synthetic, seeded):
  GPS L1 C/A   32 PRNs,  1 ms coherent (50,000-point FFT) x 40 blocks, +-5 kHz / 250 Hz (41 bins)
  GLONASS L1OF 14 FDMA channels k = -7..+6 (562.5 kHz spacing), same grid
  Galileo E1B  36 PRNs,  4 ms coherent (200,000-point FFT) x 10 blocks, +-5 kHz / 62.5 Hz (161 bins)
= 1.254e9 cells per step; one step = the 16 jobs of one capture through
ugsdr_acquire_batch.  The default line also carries a `served` section: a
bounded prefix of the configuration's Poisson request mix through the
server (p50/p99, served vs sequential ugsdr_acquire) and a short-job stream
at a load the GPU carries (--no-served skips it).  Other lines:
  --config gps_l1_4mhz | l5_weak | gal_small   other acquisition searches
  --config track         256-channel tracking bank, 10 s at 20 MHz
  --config jamming       interference stage, 400 ms at 50 MHz
  --config observables   observables + preamble search, 256 ch x 60,000 epochs
  --config dft25         the radix-25 DFT stage: CUDA-core butterfly vs tcgen05 3xTF32
  --served               the Poisson request stream through the server

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference path
(oracle/, the reference's ProcessBpsk loop with per-call FFTs) on the host
cores, on a bounded sample of the same workload, and prints the same line.
Multi-GPU: one process per GPU, each running its own replica of the
workload (jobs are independent; no collective), `scaling` = weak.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FS = 50e6
CENTER = 1590e6
SIGMA = 20.0


def log2(x):
    return math.log(x, 2)


# ------------------------------------------------------------------ workload
# Codes of every workload come from tests/golden/codes.npz, which the
# reference's own PrnGenerator::Get produced (the library's generators are
# bit-exact against it): both arms read the same chips, and the reference arm
# never loads the product library.
def golden_chips(name):
    z = np.load(ROOT / "tests" / "golden" / "codes.npz")
    n = int(z[f"{name}_len"])
    bits = np.unpackbits(z[name], axis=1)[:, :n]
    return (1.0 - 2.0 * bits).astype(np.float32)


def galileo_chips():
    return golden_chips("galileo_e1b")


def multi_workload(seed: int = 2):
    """Jobs (as plain dicts) and the synthetic int16 capture."""
    from ugsdr_gb300 import signals
    rng = np.random.default_rng(seed)
    gps = dict(enumerate(golden_chips("gps_l1ca")[:32]))
    glo = golden_chips("glonass_l1of")[0]
    e1b = galileo_chips()
    if_gps = 1575.42e6 - CENTER
    ems, planted = [], {"gps": {}, "glo": {}, "gal": {}}  # code index -> (code phase in chips, residual Doppler)
    for p in rng.choice(32, 8, replace=False):
        ph, dop = rng.uniform(0, 1023), rng.uniform(-4500, 4500)
        ems.append(signals.Emitter(gps[int(p)], 1.023e6, ph, if_gps + dop, rng.uniform(38, 48), 50.0, rng.uniform(0, 6.28)))
        planted["gps"][int(p)] = (ph, dop)
    for k in rng.choice(np.arange(-7, 7), 8, replace=False):
        f_if = 1602e6 + int(k) * 0.5625e6 - CENTER
        ph, dop = rng.uniform(0, 511), rng.uniform(-4500, 4500)
        ems.append(signals.Emitter(glo, 0.511e6, ph, f_if + dop, rng.uniform(38, 48), 50.0, rng.uniform(0, 6.28)))
        planted["glo"][int(k)] = (ph, dop)
    for p in rng.choice(36, 8, replace=False):
        ph, dop = rng.uniform(0, 8184), rng.uniform(-4500, 4500)
        ems.append(signals.Emitter(e1b[int(p)], 2.046e6, ph, if_gps + dop, rng.uniform(38, 48), 250.0, rng.uniform(0, 6.28)))
        planted["gal"][int(p)] = (ph, dop)
    raw = signals.synthesize(ems, FS, int(FS * 0.040), SIGMA, "ci16", seed + 100)
    jobs = [dict(system="gps", codes=[gps[p] for p in range(32)], n=50000, k=40, step=250.0, fe=-if_gps, if_=if_gps,
                 planted=planted["gps"], chip_rate=1.023e6)]
    for k in range(-7, 7):
        f_if = 1602e6 + k * 0.5625e6 - CENTER
        jobs.append(dict(system="glo", codes=[glo], n=50000, k=40, step=250.0, fe=-f_if, if_=f_if, letter=k,
                         planted={0: planted["glo"][k]} if k in planted["glo"] else {}, chip_rate=0.511e6))
    jobs.append(dict(system="gal", codes=[e1b[p] for p in range(36)], n=200000, k=10, step=62.5, fe=-if_gps, if_=if_gps,
                     planted=planted["gal"], chip_rate=2.046e6))
    return jobs, raw


def gal_small_workload(seed: int = 2):
    """Profiling case for the large-N kernels: the Galileo E1B job of the
    multi-constellation capture cut to 4 codes x 5 Doppler bins (200,000-point
    blocks, K = 10)."""
    jobs, raw = multi_workload(seed)
    gal = dict(jobs[-1])
    gal["codes"] = gal["codes"][:4]
    gal["step"] = 2500.0
    return [gal], raw


def gps_small_workload(seed: int = 2):
    """Profiling case for the 50,000-point kernels: the GPS job of the
    multi-constellation capture cut to 4 codes x 5 Doppler bins (K = 40)."""
    jobs, raw = multi_workload(seed)
    gps = dict(jobs[0])
    gps["codes"] = gps["codes"][:4]
    gps["step"] = 2500.0
    return [gps], raw


def gps_4mhz_workload(seed: int = 1):
    from ugsdr_gb300 import signals
    gps = dict(enumerate(golden_chips("gps_l1ca")[:32]))
    raw, _ = signals.gps_l1_config(seed=seed, codes=gps)
    jobs = [dict(system="gps", codes=[gps[p] for p in range(32)], n=4000, k=10, step=500.0, fe=0.0, if_=0.0, fs=4e6)]
    return jobs, raw


def l5_weak_workload(seed: int = 5):
    """Weak-signal GPS L5I search: real int8 at 40 MHz, IF 10 MHz, 200 ms;
    mixed and resampled to 20.46 MHz complex on the device (L = 1023, M = 2000),
    10 ms coherent (204,600-point FFT) with NH10 in the replica, x 20 blocks,
    +-5 kHz at 25 Hz (401 bins), 63 PRNs: 5.17e9 cells per search.  The
    reference's L5I table holds PRNs 1-32, so searches 33-63 reuse the codes
    of PRNs 1-31 (same work per cell)."""
    from ugsdr_gb300 import signals
    l5 = dict(enumerate(golden_chips("gps_l5i")))
    raw, _ = signals.l5_weak_config(seed, l5)
    jobs = [dict(system="l5", codes=[l5[p % 32] for p in range(63)], n=204600, k=20, step=25.0, fe=-10e6, if_=10e6,
                 fs=20.46e6, fs_in=40e6, repeats=10, sign_mask=signals.nh10_mask(), sign_segment=20460)]
    return jobs, raw


WORKLOADS = {"multi": multi_workload, "gps_l1_4mhz": gps_4mhz_workload, "gal_small": gal_small_workload,
             "gps_small": gps_small_workload, "l5_weak": l5_weak_workload}
WORKLOAD_DESC = {
    "multi": "multi-constellation batch: int16 I/Q 50 MHz 40 ms; GPS L1 C/A 32x41x50000x40, "
             "GLONASS L1OF 14ch x41x50000x40, Galileo E1B 36x161x200000x10",
    "gps_l1_4mhz": "GPS L1 C/A int8 4 MHz 10 ms; 32 PRN x 21 Doppler x 4000 x 10",
    "gal_small": "Galileo E1B 4 codes x 5 Doppler x 200000 x 10 (profiling case)",
    "gps_small": "GPS L1 C/A 4 codes x 5 Doppler x 50000 x 40 (profiling case)",
    "l5_weak": "GPS L5I weak-signal: real int8 IF 40 MHz 200 ms -> 20.46 MHz complex on device; "
               "63 PRN x 401 Doppler x 204600 (10 ms, NH10 wiped) x 20",
}


def sample_type_of(raw):
    from ugsdr_gb300 import _lib as L
    if raw.ndim == 1:
        return L.SAMPLES_RI8
    return L.SAMPLES_CI16 if raw.dtype == np.int16 else L.SAMPLES_CI8


def oracle_code(pyoracle, j, chips):
    """The job's replica as the reference builds it: RepeatCodeNTimes +
    SequentialUpsampler (fse.hpp:295), then the per-period signs."""
    reps = j.get("repeats", 1)
    code = pyoracle.upsample(np.tile(chips, reps), j["n"])
    seg = j.get("sign_segment", 0)
    for s in range(32):
        if (j.get("sign_mask", 0) >> s) & 1:
            code[s * seg:(s + 1) * seg] *= -1
    return code


def n_doppler(step, rng=5000.0):
    n, d = 0, -rng
    while d <= rng:
        n += 1
        d += step
    return n


def job_cells(j):
    return len(j["codes"]) * n_doppler(j["step"]) * j["n"]


def inverse_flops(j):
    """Algorithmic flops of the inverse stage: per (code, Doppler, block) one
    N-point IFFT (5 N log2 N) + conj-multiply and |.| accumulate (10 N)."""
    n = j["n"]
    return len(j["codes"]) * n_doppler(j["step"]) * j["k"] * (5 * n * log2(n) + 10 * n)


# DRAM bytes per inverse-transform point of the four-step kernels (inv_rows +
# inv_cols), measured with ncu on the 200,000-point profiling case (16.1: the
# intermediate B buffer is 16 of it); see profiles/.
TRAFFIC_BYTES_PER_INVERSE_POINT = 16.1


def inverse_points(j):
    return len(j["codes"]) * n_doppler(j["step"]) * j["k"] * j["n"]


def inverse_bytes(j):
    """Algorithmic HBM bytes of the inverse stage: one-sided spectra read once
    per (Doppler, block) row, code spectra once, 16 B per cell record."""
    n, nd = j["n"], n_doppler(j["step"])
    return nd * j["k"] * (n // 2 + 1) * 8 + len(j["codes"]) * (n // 2 + 1) * 8 + len(j["codes"]) * nd * 16


# ------------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self):
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200", "-i", str(int(os.environ.get("LOCAL_RANK", 0)))],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) > 8 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ------------------------------------------------------------------ ours arm
def run_ours(args, world, rank):
    import torch
    from ugsdr_gb300 import _lib as L
    from ugsdr_gb300 import api

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    jobs, raw = WORKLOADS[args.config]()
    fs = jobs[0].get("fs", FS)
    stype = sample_type_of(raw)
    ctx = api.Context(dev)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    handles = []
    for j in jobs:
        hs = [ctx.code_put(c, j["n"], repeats=j.get("repeats", 1), sign_mask=j.get("sign_mask", 0),
                           sign_segment=j.get("sign_segment", 0)) for c in j["codes"]]
        handles.append(hs)
    # inputs resident in HBM for `value`; pinned host copy for `e2e`
    d_raw = torch.from_numpy(raw.copy()).cuda(dev)
    h_raw = torch.empty(raw.shape, dtype=d_raw.dtype, pin_memory=True)
    h_raw.copy_(torch.from_numpy(raw))
    h_np = h_raw.numpy()
    n_samples = raw.shape[0]

    def mk(on_device):
        out = []
        for j, hs in zip(jobs, handles):
            src = d_raw.data_ptr() if on_device else h_np
            fs_in = j.get("fs_in", 0.0)
            out.append(ctx.make_job(src, stype, fs, j["n"], j["k"], hs, 5000.0, j["step"], n_samples=n_samples,
                                    on_device=on_device, frontend_frequency=j["fe"], intermediate_frequency=j["if_"],
                                    input_sampling_rate=fs_in, code_offset_ratio=(fs_in / fs) if fs_in else 1.0))
        return out

    dev_jobs, host_jobs = mk(True), mk(False)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")  # > L2 (129 MB)
    cells = sum(job_cells(j) for j in jobs)

    # four-step tile shapes: measured by the autotuner on this workload's jobs
    # (Doppler grids cut), before the warm-up and outside the timed region
    t0 = time.perf_counter()
    tried = [] if args.no_tune else ctx.autotune(dev_jobs)
    tune_s = time.perf_counter() - t0
    tiles = {}
    for n in sorted({j["n"] for j in jobs if j["n"] > 12000}):
        t = ctx.tile_shape(n)
        rule_ms = next((x["ms"] for x in tried if x["block_samples"] == n), None)
        key = ("n1", "cols", "rows", "warp_cols", "warp_rows")
        kept_ms = next((x["ms"] for x in tried if x["block_samples"] == n and all(x[k] == t[k] for k in key)), None)
        tiles[str(n)] = {"split": f"{t['n1']}x{n // t['n1']}", "cols": t["cols"], "rows": t["rows"],
                         "column_kernel": "warp-owned" if t["warp_cols"] else "tile",
                         "row_kernel": {0: "tile", 1: "warp-owned", 2: "warp-owned, 3 rows/warp, code via L2"}[t["warp_rows"]],
                         "shapes_timed": sum(1 for x in tried if x["block_samples"] == n),
                         "rule_ms": rule_ms, "kept_ms": kept_ms}

    for _ in range(args.warmup):
        ctx.acquire_batch(dev_jobs)
    torch.cuda.synchronize()

    def timed(job_list, k, with_timing):
        times = []
        launches0 = ctx.launch_count()
        if with_timing:
            ctx.reset_timing()
            ctx.enable_timing(True)
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.zero_()  # L2 flush between steps, outside the events
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            stream.synchronize()
            s.record(stream)
            t0 = time.perf_counter()
            ctx.acquire_batch(job_list)
            e.record(stream)
            e.synchronize()
            wall = time.perf_counter() - t0
            times.append(max(s.elapsed_time(e) / 1e3, wall))
        ctx.enable_timing(False)
        return times, (ctx.launch_count() - launches0) / k

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler() as clk:
        times, launches = timed(dev_jobs, args.steps, True)
    torch.cuda.synchronize()
    t_step = float(np.mean(times))
    if world > 1:
        t = torch.tensor([t_step], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
    inv_name = "acq_inverse_large" if jobs[0]["n"] > 12000 else "acq_inverse"
    n_inv, ms_inv = ctx.kernel_time(inv_name)
    n_fwd, ms_fwd = ctx.kernel_time(inv_name.replace("inverse", "forward"))
    flops_inv = sum(inverse_flops(j) for j in jobs) * args.steps
    bytes_inv = sum(inverse_bytes(j) for j in jobs) * args.steps
    large = all(j["n"] > 12000 for j in jobs)  # four-step kernels (the measured traffic applies)
    traffic = (TRAFFIC_BYTES_PER_INVERSE_POINT * sum(inverse_points(j) for j in jobs) * args.steps / max(n_inv, 1)
               if large else None)

    # end to end through the C ABI with pinned host samples
    e2e_times, _ = timed(host_jobs, max(2, args.steps // 2), False)
    t_e2e = float(np.mean(e2e_times))
    h2d = raw.nbytes  # one upload per step (jobs share the capture)
    n_cells_rec = sum(len(j["codes"]) * n_doppler(j["step"]) for j in jobs)
    d2h = n_cells_rec * 16

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s: SMs x 128 FP32 lanes x FMA x clock
    achieved = flops_inv / (ms_inv / 1e3) / 1e12 if ms_inv > 0 else None
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    hbm_ach = bytes_inv / (ms_inv / 1e3) / 1e9 if ms_inv > 0 else None
    clocks = clk.summary()
    line = {
        "metric": "acq cells/s (PRN x Doppler x code-phase)",
        "value": world * cells / t_step,
        "unit": "cells/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_step * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded int16/int8 I/Q captures; Galileo E1B chips from the reference's code tables)",
        "config": {"workload": WORKLOAD_DESC[args.config],
                   "cells_per_step": cells, "jobs_per_step": len(jobs), "parallelism": f"replicas x{world}",
                   "l2": "flushed between steps (256 MB write); working set > L2",
                   "tiles": {"chosen_by": "rule (--no-tune)" if args.no_tune else
                             f"ugsdr_autotune ({len(tried)} shapes timed in {tune_s:.1f} s before the warm-up)",
                             **tiles}},
        "e2e": {"value": world * cells / t_e2e, "unit": "cells/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": t_e2e * 1e3},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32", "kernel": inv_name, "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak if achieved else None, "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read+write per inverse point (16.1 B, 200k profiling "
                                       "case) x points per launch" if traffic else None,
                     "algorithmic_bytes_per_launch": bytes_inv / max(n_inv, 1),
                     "peak_source": f"{n_sm} SMs x 128 FP32 lanes x 2 x sm_max_mhz {sm_max} (MEASURED_PEAKS.json)",
                     "launches": n_inv, "avg_launch_ms": ms_inv / max(n_inv, 1),
                     "hbm": {"achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s",
                             "frac": hbm_ach / hbm_peak if hbm_ach else None},
                     "forward_ms_share": ms_fwd / (ms_fwd + ms_inv) if ms_inv else None},
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, jobs, raw, fs)
    if rank == 0 and world == 1 and args.config == "multi" and not args.no_served:
        line["served"] = served_section()
    return line


# ------------------------------------------------------------- served stream
def served_requests(seed: int, n_req: int, rate: float = 2000.0):
    """Seeded request stream: fs in {2.046, 4, 10.23, 20.46, 50} MHz, coherent
    1-20 ms, K 1-40, 1-63 codes of GPS L1 C/A, L5I or Galileo E1B (as many as
    the system has), Doppler +-5 kHz at 1/(2 T), int8 or int16, 0-12 signals
    at 35-50 dB-Hz; Poisson arrivals at 2000 req/s.  Captures are synthesised
    once per sampling rate (long enough for the largest request) and each
    request reads its own window."""
    from ugsdr_gb300 import _lib as L
    from ugsdr_gb300 import api
    rng = np.random.default_rng(seed)
    systems = {"gps": (list(golden_chips("gps_l1ca")), 1.023e6, 1),
               "l5i": (list(golden_chips("gps_l5i")), 10.23e6, 1),
               "e1b": (list(galileo_chips()), 2.046e6, 4)}
    rates = [2.046e6, 4e6, 10.23e6, 20.46e6, 50e6]
    reqs, t = [], 0.0
    for _ in range(n_req):
        t += rng.exponential(1 / rate)
        sysname = ["gps", "l5i", "e1b"][rng.integers(3)]
        chips, chip_rate, period_ms = systems[sysname]
        fs = rates[rng.integers(len(rates))]
        if fs <= chip_rate:  # the code must be oversampled
            fs = rates[-1]
        t_ms = int(rng.integers(1, 21))
        t_ms = max(period_ms, t_ms // period_ms * period_ms)
        k = int(rng.integers(1, 41))
        n_codes = int(rng.integers(1, 64))
        codes = [int(c) for c in rng.choice(len(chips), size=min(n_codes, len(chips)), replace=False)]
        reqs.append(dict(arrival=t, system=sysname, fs=fs, t_ms=t_ms, k=k, codes=codes, step=1000.0 / (2 * t_ms),
                         stype="ci8" if rng.integers(2) else "ci16", n_sig=int(rng.integers(0, 13))))
    return reqs, systems


def run_short_stream(ctx, n_req: int = 200, rate: float = 200.0, seed: int = 9, background: int = 0):
    """Latency at a load the GPU can carry: a Poisson stream of short GPS L1
    C/A searches (int8 I/Q at 4 MHz, 1 ms x 4 blocks, 8 PRNs, +-5 kHz at
    500 Hz: 672,000 cells each) through the server, against the same search
    run alone through ugsdr_acquire.  background: that many long searches
    (GPS L1 C/A at 50 MHz, 32 PRNs x 161 Doppler bins x 50,000 x 40 blocks,
    1.03e10 cells, ~0.8 s each) submitted just before the stream starts, more
    than the server's general slots."""
    from ugsdr_gb300 import _lib as L
    from ugsdr_gb300 import api, signals
    rng = np.random.default_rng(seed)
    gps = golden_chips("gps_l1ca")
    raw, _ = signals.gps_l1_config(seed=seed, codes={p: gps[p] for p in range(32)}, fs=4e6, ms=4, visible=4)
    bg_job, bg_handles = None, []
    if background:
        bg_raw, _ = signals.gps_l1_config(seed=seed + 1, codes={p: gps[p] for p in range(32)}, fs=50e6, ms=40,
                                          sample_type="ci16")
        bg_handles = [ctx.code_put(gps[p], 50000) for p in range(32)]
        bg_job = ctx.make_job(bg_raw, L.SAMPLES_CI16, 50e6, 50000, 40, bg_handles, 5000.0, 62.5)
    jobs, handles = [], []
    for _ in range(n_req):
        prns = rng.choice(32, 8, replace=False)
        hs = [ctx.code_put(gps[int(p)], 4000) for p in prns]
        handles += hs
        jobs.append(ctx.make_job(raw, L.SAMPLES_CI8, 4e6, 4000, 4, hs, 5000.0, 500.0))
    cells = 8 * n_doppler(500.0) * 4000
    for j in jobs[:5]:
        ctx.acquire(j)
    t0 = time.perf_counter()
    for j in jobs[:50]:
        ctx.acquire(j)
    alone_ms = (time.perf_counter() - t0) / 50 * 1e3
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    srv = api.Server(ctx, max_inflight=4, policy=L.SERVE_RESPONSE_RATIO)
    if background:
        # steady state: the general slots' scratch already grown by earlier long
        # searches (a cold slot's first multi-GB allocation holds the admission
        # thread for ~0.1 s)
        for t in [srv.submit(bg_job) for _ in range(background)]:
            while srv.poll(t) is None:
                time.sleep(0.001)
    bg_tickets = [srv.submit(bg_job) for _ in range(background)]
    t0 = time.perf_counter()
    tickets, done_at, i = [], {}, 0
    while len(done_at) < n_req:
        now = time.perf_counter() - t0
        while i < n_req and arrivals[i] <= now:
            tickets.append(srv.submit(jobs[i]))
            i += 1
        for k, t in enumerate(tickets):
            if k not in done_at and srv.poll(t) is not None:
                done_at[k] = time.perf_counter() - t0
        time.sleep(0.0002)
    bg_busy = sum(1 for t in bg_tickets if srv.poll(t) is None)  # long searches still on the server at the end
    srv.close()
    for h in handles + bg_handles:
        ctx.code_release(h)
    lat = np.array([done_at[k] - arrivals[k] for k in range(n_req)]) * 1e3
    out = {"workload": "GPS L1 C/A int8 4 MHz, 1 ms x 4 blocks, 8 PRNs, 21 Doppler bins (672,000 cells) per request",
           "requests": n_req, "rate_req_s": rate, "p50_ms": float(np.percentile(lat, 50)),
           "p99_ms": float(np.percentile(lat, 99)), "alone_ms": alone_ms,
           "cells_s": n_req * cells / (max(done_at.values()) - arrivals[0])}
    if background:
        out["background"] = (f"{background} long searches (GPS L1 C/A 50 MHz int16, 32 PRNs x 161 bins x 50,000 x 40 "
                             f"blocks, 1.03e10 cells each) submitted at the start, after {background} more had grown "
                             f"the slots' scratch; {bg_busy} still running when the last short search returned")
    return out


def served_section():
    """The served half of the metric beside the default line: the
    configuration's request mix (a bounded prefix of the seeded Poisson
    stream at 2000 req/s) served vs the same requests one after another
    through ugsdr_acquire, and the short-job stream's latency."""
    from argparse import Namespace
    from ugsdr_gb300 import api
    mix = run_served(Namespace(requests=8, rate=2000.0, inflight=4, policy="response_ratio"))
    ctx = api.Context(0)
    try:
        short = run_short_stream(ctx)
        loaded = run_short_stream(ctx, background=12)
    finally:
        ctx.close()
    keep = ("value", "requests", "p50_ms", "p99_ms", "offered_load", "sequential_cells_s", "served_over_sequential",
            "max_inflight_seen", "wall_s")
    return {"mix": {k: mix[k] for k in keep}, "short_jobs": short, "short_jobs_under_load": loaded,
            "note": "p99 < 20 ms at 2000 req/s of the configuration's mix (mean 3.4e9 cells per request) would need "
                    "~7e12 cells/s; the short-job stream shows the latency the server gives at a feasible load"}


def run_served(args):
    import torch
    from ugsdr_gb300 import _lib as L
    from ugsdr_gb300 import api, signals
    n_req = args.requests
    reqs, systems = served_requests(7, n_req, args.rate)
    torch.cuda.set_device(0)
    ctx = api.Context(0)
    rng = np.random.default_rng(8)
    captures = {}
    for fs in sorted({r["fs"] for r in reqs}):
        need = max(int(fs * r["t_ms"] / 1000) * r["k"] for r in reqs if r["fs"] == fs)
        ems = []
        for _ in range(4):
            sysname = ["gps", "l5i", "e1b"][rng.integers(3)]
            chips, rate, _ = systems[sysname]
            if rate >= fs:
                continue
            ems.append(signals.Emitter(chips[rng.integers(len(chips))], rate, rng.uniform(0, len(chips[0])),
                                       rng.uniform(-4500, 4500), rng.uniform(35, 50)))
        raw16 = signals.synthesize(ems, fs, need, SIGMA, "ci16", int(fs) % 1000)
        captures[fs] = {"ci16": raw16, "ci8": np.clip(raw16, -128, 127).astype(np.int8)}
    handles = {}

    def code_handle(sysname, c, n, t_ms):
        key = (sysname, c, n)
        if key not in handles:
            chips, rate, period_ms = systems[sysname]
            handles[key] = ctx.code_put(chips[c], n, repeats=t_ms // period_ms)
        return handles[key]

    jobs, cells = [], []
    for r in reqs:
        n = int(r["fs"] * r["t_ms"] / 1000)
        hs = [code_handle(r["system"], c, n, r["t_ms"]) for c in r["codes"]]
        raw = captures[r["fs"]][r["stype"]][: n * r["k"]]
        st = L.SAMPLES_CI8 if r["stype"] == "ci8" else L.SAMPLES_CI16
        jobs.append(ctx.make_job(raw, st, r["fs"], n, r["k"], hs, 5000.0, r["step"]))
        cells.append(len(hs) * n_doppler(r["step"]) * n)

    # served: Poisson arrivals into the continuous-batching server
    policy = {"fifo": L.SERVE_FIFO, "response_ratio": L.SERVE_RESPONSE_RATIO}[args.policy]
    srv = api.Server(ctx, max_inflight=args.inflight, policy=policy)
    warm = srv.submit(jobs[0])
    srv.drain()
    srv.poll(warm)
    t0 = time.perf_counter()
    tickets, done_at, failures = [], {}, []
    i = 0
    while len(done_at) < len(jobs):
        now = time.perf_counter() - t0
        while i < len(jobs) and reqs[i]["arrival"] <= now:
            tickets.append(srv.submit(jobs[i]))
            i += 1
        for k, t in enumerate(tickets):
            if k in done_at:
                continue
            try:
                finished = srv.poll(t) is not None
            except L.UgsdrError as e:  # a failed request still completes (with its error)
                failures.append({"request": k, "error": str(e)})
                finished = True
            if finished:
                done_at[k] = time.perf_counter() - t0
        time.sleep(0.0002)
    t_total = max(done_at.values()) - reqs[0]["arrival"]
    lat = np.array([done_at[k] - reqs[k]["arrival"] for k in range(len(jobs))]) * 1e3
    stats = srv.stats()
    srv.close()
    served = sum(cells) / t_total

    # sequential: the same jobs one after another through ugsdr_acquire (no overlap)
    t1 = time.perf_counter()
    for j in jobs:
        ctx.acquire(j)
    t_seq = time.perf_counter() - t1

    # plain: one (code, Doppler) search per call through the per-op entries,
    # the reference's ProcessBpsk structure on the GPU policies; bounded sample
    r = min(range(len(reqs)), key=lambda k: cells[k])
    req = reqs[r]
    n = int(req["fs"] * req["t_ms"] / 1000)
    x = captures[req["fs"]][req["stype"]][: n * req["k"]].astype(np.float32)
    x = (x[:, 0] + 1j * x[:, 1]).astype(np.complex64)
    chips, rate, period_ms = systems[req["system"]]
    grid = [-5000.0 + d * req["step"] for d in range(n_doppler(req["step"]))]
    t2 = time.perf_counter()
    rows = 0
    for c in req["codes"][:2]:
        code = api.repeat_upsample(chips[c], req["t_ms"] // period_ms, n)
        spec = ctx.prepare_code_spectrum(code)
        for d in grid[:3]:
            y = ctx.mix(x.copy(), req["fs"], -d)
            acc = np.zeros(n, np.float32)
            for b in range(req["k"]):
                acc += ctx.abs(ctx.filter_optimized(y[b * n:(b + 1) * n], spec))
            ctx.max_index(acc)
            ctx.mean_stddev(acc)
            rows += 1
    plain = rows * n / (time.perf_counter() - t2)
    return {
        "metric": "served acq cells/s (continuous batching) with p50/p99 latency",
        "value": served, "unit": "cells/s", "n_gpus": 1, "requests": len(jobs),
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "offered_rate_req_s": args.rate, "wall_s": t_total, "max_inflight_seen": stats["max_inflight_seen"],
        "offered_load": args.rate * float(np.mean(cells)) / (sum(cells) / t_seq),
        "failed_requests": failures,
        "per_request": [{"arrival_ms": round(reqs[k]["arrival"] * 1e3, 2), "cell_blocks": int(cells[k] * reqs[k]["k"]),
                         "latency_ms": round(float(lat[k]), 1)} for k in range(len(jobs))],
        "sequential_cells_s": sum(cells) / t_seq, "plain_cells_s": plain, "served_over_plain": served / plain,
        "served_over_sequential": served / (sum(cells) / t_seq),
        "plain_sample": f"{rows} (code, Doppler) rows of a {n}-sample x {req['k']}-block request, per-op entries",
        "config": {"workload": f"served stream: Poisson {args.rate:g} req/s, fs {{2.046,4,10.23,20.46,50}} MHz, Tcoh 1-20 ms, "
                               "K 1-40, 1-63 codes of L1 C/A / L5I / E1B, int8/int16", "inflight": args.inflight,
                   "policy": args.policy,
                   "cells_total": int(sum(cells))},
    }


# ------------------------------------------------------------ tracking bank
TRACK_FS = 20e6
TRACK_FLOPS_PER_CHANNEL_SAMPLE = 26  # carrier wipe-off 6 + five taps x (I, Q) x FMA 2
TRACK_OUT_BYTES = 88                 # ugsdr_track_output per channel-epoch


def track_capture(dev, seconds, seed=3, n_channels=256, sigma=20.0):
    """256-channel tracking input, synthesised on the device in float64 phase
    (10 s at 20 MHz is 2e8 int16 I/Q samples): 12 GPS L1 C/A and 12 Galileo E1
    emitters (E1B data at 250 sps and E1C pilot, BOC(1,1), half the power
    each), Doppler +-5 kHz with a 0.5 Hz/s ramp, C/N0 35-50 dB-Hz, AWGN sigma
    20 LSB.  Channels: the 36 signal channels (GPS, E1B, E1C) started at the
    true code phase and initial Doppler, then channels on the other codes
    (random phase and Doppler) up to n_channels.  Returns the device capture,
    the channel list and the code table."""
    import torch
    from ugsdr_gb300 import _lib as L
    from ugsdr_gb300 import api
    rng = np.random.default_rng(seed)
    fs = TRACK_FS
    device = f"cuda:{dev}" if isinstance(dev, int) else dev
    gps = list(golden_chips("gps_l1ca")[:32])
    e1b, e1c = golden_chips("galileo_e1b"), golden_chips("galileo_e1c")
    codes = gps + list(e1b) + list(e1c)
    rate_of = [1.023e6] * 32 + [2.046e6] * 100
    ems = []
    for p in rng.choice(32, 12, replace=False):
        ems.append(dict(parts=[(int(p), 1.0, 50.0)], rate=1.023e6, delay=rng.uniform(0, 1023),
                        f0=rng.uniform(-5000, 5000), cn0=rng.uniform(35, 50), phi=rng.uniform(0, 1)))
    for p in rng.choice(50, 12, replace=False):
        h = 1 / np.sqrt(2)
        ems.append(dict(parts=[(32 + int(p), h, 250.0), (82 + int(p), -h, 0.0)], rate=2.046e6,
                        delay=rng.uniform(0, 8184), f0=rng.uniform(-5000, 5000), cn0=rng.uniform(35, 50),
                        phi=rng.uniform(0, 1)))
    n = int(fs * seconds)
    cap = torch.empty((n, 2), dtype=torch.int16, device=device)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    code_t = [torch.tensor(c, device=device) for c in codes]
    bits = {}
    chunk = 10_000_000
    for a in range(0, n, chunk):
        m = min(chunk, n - a)
        t = (a + torch.arange(m, dtype=torch.float64, device=device)) / fs
        re = torch.zeros(m, dtype=torch.float32, device=device)
        im = torch.zeros_like(re)
        for k, e in enumerate(ems):
            amp = sigma * np.sqrt(2.0 * 10 ** (e["cn0"] / 10.0) / fs)
            pos = t * (e["rate"] * (1 + e["f0"] / 1575.42e6)) - e["delay"]
            sig = torch.zeros_like(re)
            for j, (ci, w, drate) in enumerate(e["parts"]):
                c = code_t[ci]
                chip = torch.remainder(torch.floor(pos), len(codes[ci])).long()
                part = c[chip] * w
                if drate > 0:
                    key = (k, j)
                    if key not in bits:
                        nb = int(seconds * drate) + 4
                        bits[key] = torch.tensor(rng.choice([-1.0, 1.0], size=nb).astype(np.float32), device=device)
                    part = part * bits[key][torch.floor(t * drate).long() + 1]
                sig += part
            cyc = e["f0"] * t + 0.25 * t * t + e["phi"]  # 0.5 Hz/s ramp
            ang = (2 * np.pi * (cyc - torch.floor(cyc))).float()
            re += amp * sig * torch.cos(ang)
            im += amp * sig * torch.sin(ang)
        noise = torch.randn((m, 2), generator=gen, device=device) * sigma
        x = torch.stack([re, im], dim=1) + noise
        cap[a:a + m] = torch.clamp(torch.round(x), -32768, 32767).to(torch.int16)
        del t, re, im, noise, x
    chans = []
    for e in ems:
        for ci, _, _ in e["parts"]:
            period = len(codes[ci]) / rate_of[ci]  # s
            cp = (e["delay"] / e["rate"] * fs) % (period * fs)
            chans.append(dict(code=ci, fs=fs, code_frequency=rate_of[ci], code_phase=float(round(cp)),
                              carrier_frequency=e["f0"], boc=int(ci >= 32)))
    used = {c["code"] for c in chans}
    others = [c for c in range(len(codes)) if c not in used]
    i = 0
    while len(chans) < n_channels:
        ci = others[i % len(others)]
        i += 1
        period = len(codes[ci]) / rate_of[ci]
        chans.append(dict(code=ci, fs=fs, code_frequency=rate_of[ci], code_phase=float(rng.integers(0, int(period * fs))),
                          carrier_frequency=rng.uniform(-5000, 5000), boc=int(ci >= 32)))
    return cap, chans, codes


TRACK_CFG = dict(early_late=0.15, very_early_late=0.5, pll_bw=15.0, dll_bw=1.0, fll_bw=0.0)


def track_cpu_baseline(cap, chans, codes, threads=None, epochs=2000):
    """FP64 oracle channel loop (oracle/track_oracle.cpp) on the host cores:
    one channel per thread over `epochs` ms of the capture."""
    from concurrent.futures import ThreadPoolExecutor
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    threads = threads or os.cpu_count() or 1
    spm = int(TRACK_FS / 1000)
    raw = cap[: spm * epochs].cpu().numpy().astype(np.float32)
    x = (raw[:, 0] + 1j * raw[:, 1]).astype(np.complex64)
    sel = chans[:threads]

    def one(ch):
        return pyoracle.track(x, spm, epochs, codes[ch["code"]], TRACK_FS, ch["code_frequency"], ch["code_phase"],
                              ch["carrier_frequency"], **TRACK_CFG)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(one, sel))
    dt = time.perf_counter() - t0
    return {"value": len(sel) * spm * epochs / dt, "unit": "channel-samples/s", "cores": threads, "kind": "port",
            "sample": f"{len(sel)} channels x {epochs} epochs of the same capture in {dt:.2f}s "
                      "(FP64 oracle loop, one channel per thread)"}


def run_track(args, world, rank):
    """Tracking correlator bank: 256 channels over `--track-seconds` (default
    10 s) of 20 MHz int16 I/Q per step; one step = one ugsdr_track_run of the
    whole capture on a freshly created bank."""
    import torch
    from ugsdr_gb300 import _lib as L
    from ugsdr_gb300 import api
    if args.impl == "reference" and rank != 0:
        return None
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    seconds = args.track_seconds
    cap, chans, codes = track_capture(dev, seconds)
    n_epochs = int(round(seconds * 1000))
    spm = int(TRACK_FS / 1000)
    nch = len(chans)
    if args.impl == "reference":
        if rank != 0:
            return None
        vals = [track_cpu_baseline(cap, chans, codes) for _ in range(args.warmup + args.steps)][args.warmup:]
        v = float(np.mean([b["value"] for b in vals]))
        return {"metric": "tracking channel-samples/s", "value": v, "unit": "channel-samples/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": nch * n_epochs * spm / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "impl": "reference", "config": {"workload": f"tracking bank {nch} ch, 20 MHz int16, {seconds} s"},
                "cpu_baseline": {k: vals[-1][k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": v, "unit": "channel-samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    ctx = api.Context(dev)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    d_out = torch.empty(n_epochs * nch * TRACK_OUT_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    h_cap = torch.empty(cap.shape, dtype=cap.dtype, pin_memory=True)
    h_cap.copy_(cap)
    h_out = torch.empty(n_epochs * nch * TRACK_OUT_BYTES, dtype=torch.uint8, pin_memory=True)
    h_out_np = h_out.numpy().view(api.TRACK_DTYPE).reshape(n_epochs, nch)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    def bank():
        return api.TrackBank(ctx, chans, codes, **TRACK_CFG)

    def step(b, on_device):
        if on_device:
            b.run_device(cap.data_ptr(), L.SAMPLES_CI16, n_epochs, d_out.data_ptr())
        else:
            b.run(h_cap.numpy(), L.SAMPLES_CI16, n_epochs, out=h_out_np)

    for _ in range(args.warmup):
        b = bank()
        step(b, True)
        torch.cuda.synchronize()
        b.close()

    def timed(k, on_device):
        times = []
        l0 = ctx.launch_count()
        for _ in range(k):
            b = bank()
            with torch.cuda.stream(stream):
                flush.zero_()
            stream.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            t0 = time.perf_counter()
            step(b, on_device)
            e.record(stream)
            e.synchronize()
            times.append(max(s.elapsed_time(e) / 1e3, time.perf_counter() - t0 if not on_device else 0.0))
            b.close()
        return times, (ctx.launch_count() - l0) / k

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler() as clk:
        times, launches = timed(args.steps, True)
    t_step = float(np.mean(times))
    if world > 1:
        t = torch.tensor([t_step], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
    e2e_times, _ = timed(max(2, args.steps // 2), False)
    t_e2e = float(np.mean(e2e_times))
    ch_samples = nch * n_epochs * spm
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_max * 1e6 / 1e12
    achieved = ch_samples * TRACK_FLOPS_PER_CHANNEL_SAMPLE / t_step / 1e12
    alg_bytes = n_epochs * spm * 4 + n_epochs * nch * TRACK_OUT_BYTES
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    line = {
        "metric": "tracking channel-samples/s", "value": world * ch_samples / t_step, "unit": "channel-samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 loops)",
        "data": "synthetic (device-synthesised int16 I/Q, seeded)",
        "config": {"workload": f"tracking bank: {nch} channels (GPS L1 C/A + Galileo E1B/E1C BOC(1,1)), VE/E/P/L/VL "
                               f"0.5/0.15 chip, PLL 15 Hz, DLL 1 Hz, 1 ms epochs; int16 I/Q 20 MHz, {seconds} s",
                   "real_time_factor": seconds / t_step, "channels": nch, "epochs": n_epochs,
                   "parallelism": f"replicas x{world}", "l2": "flushed between steps (256 MB write); input 800 MB > L2"},
        "e2e": {"value": world * ch_samples / t_e2e, "unit": "channel-samples/s", "h2d_bytes_per_step": int(cap.numel() * 2),
                "d2h_bytes_per_step": n_epochs * nch * TRACK_OUT_BYTES, "ms_per_step": t_e2e * 1e3},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32", "kernel": "track_bank", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": None,
                     "flops_per_channel_sample": TRACK_FLOPS_PER_CHANNEL_SAMPLE,
                     "peak_source": f"{n_sm} SMs x 128 FP32 lanes x 2 x sm_max_mhz {sm_max} (MEASURED_PEAKS.json)",
                     "hbm": {"achieved": alg_bytes / t_step / 1e9, "peak": hbm_peak, "unit": "GB/s",
                             "frac": alg_bytes / t_step / 1e9 / hbm_peak}},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = track_cpu_baseline(cap, chans, codes)
    return line


# ------------------------------------------------------- interference stage
JAM_FS = 50e6
JAM_SECONDS = 0.4
JAM_BIN = 20  # CW jammer on STFT bin 20 (7.8125 MHz at 50 MHz)
# algorithmic bytes per sample: the detector reads the samples once and writes
# 8 rounds x (1 B bin + 8 B J/N) per 32-sample hop; the wideband filter reads
# and writes them once; the in-place copy back reads and writes them once
JAM_DETECT_BYTES = 8 + 8 * 9 / 32
JAM_WIDEBAND_BYTES = 16
JAM_COPY_BYTES = 16


def jamming_capture(dev, seconds=JAM_SECONDS):
    """Complex float samples at 50 MHz: noise (sigma 0.5 per part) + a CW
    jammer of amplitude 10 on an STFT bin centre, synthesised on the device
    from a fixed seed."""
    import torch
    n = int(round(seconds * JAM_FS))
    gen = torch.Generator(device=f"cuda:{dev}")
    gen.manual_seed(5)
    x = torch.randn((n, 2), generator=gen, device=f"cuda:{dev}") * 0.5
    t = torch.arange(n, device=f"cuda:{dev}", dtype=torch.float64)
    ph = 2 * np.pi * (JAM_BIN / 128) * t
    x[:, 0] += (10 * torch.cos(ph)).float()
    x[:, 1] += (10 * torch.sin(ph)).float()
    return x.contiguous()


def jamming_cpu_baseline(x_host, samples=2_000_000):
    """JammingSuppressionEngine::Process restated in the oracle (FP64-internal
    FFT, float arithmetic), one thread, on the first `samples` samples."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    xs = x_host[:samples]
    t0 = time.perf_counter()
    det, _ = pyoracle.jamming(xs, JAM_FS)
    dt = time.perf_counter() - t0
    return {"value": len(xs) / dt, "unit": "samples/s", "cores": 1, "kind": "port",
            "sample": f"{len(xs)} samples (first {len(xs) / JAM_FS * 1e3:.0f} ms) in {dt:.2f}s, "
                      f"{len(det)} detections (oracle engine, one thread)"}


def run_jamming(args, world, rank):
    """Interference stage: JammingSuppressionEngine<complex<float>>(50 MHz)
    .Process over 400 ms of samples per step (detect + wideband suppression,
    in place on the device)."""
    import torch
    from ugsdr_gb300 import api
    if args.impl == "reference" and rank != 0:
        return None
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    pristine = jamming_capture(dev)
    n = pristine.shape[0]
    workload = (f"interference stage: JammingSuppressionEngine::Process (STFT 128/96 detection + wideband "
                f"suppression), complex float {JAM_FS / 1e6:.0f} MHz, {JAM_SECONDS * 1e3:.0f} ms, CW jammer + noise")
    if args.impl == "reference":
        xh = pristine.cpu().numpy().view(np.complex64).ravel()
        vals = [jamming_cpu_baseline(xh) for _ in range(args.warmup + args.steps)][args.warmup:]
        v = float(np.mean([b["value"] for b in vals]))
        return {"metric": "interference stage samples/s", "value": v, "unit": "samples/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": n / v * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
                "config": {"workload": workload},
                "cpu_baseline": {k: vals[-1][k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": v, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    ctx = api.Context(dev)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    work = torch.empty_like(pristine)
    h_pristine = pristine.cpu().numpy().view(np.complex64).ravel().copy()
    h_work = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy().view(np.complex64).ravel()

    def timed(k, on_device):
        times, dets = [], None
        l0 = ctx.launch_count()
        for _ in range(k):
            if on_device:
                with torch.cuda.stream(stream):
                    work.copy_(pristine)
            else:
                np.copyto(h_work, h_pristine)
            stream.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            t0 = time.perf_counter()
            if on_device:
                dets = ctx.jamming_suppress(work.data_ptr(), JAM_FS, n=n)
            else:
                dets = ctx.jamming_suppress(h_work, JAM_FS)
            e.record(stream)
            e.synchronize()
            times.append(max(s.elapsed_time(e) / 1e3, time.perf_counter() - t0))
        return times, (ctx.launch_count() - l0) / k, dets

    timed(args.warmup, True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ctx.enable_timing(True)
    ctx.reset_timing()
    with ClockSampler() as clk:
        times, launches, dets = timed(args.steps, True)
    kt = {name: ctx.kernel_time(name) for name in ("jam_stft_detect", "jam_wideband")}
    ctx.enable_timing(False)
    t_step = float(np.mean(times))
    if world > 1:
        t = torch.tensor([t_step], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
    e2e_times, _, _ = timed(max(2, args.steps // 2), False)
    t_e2e = float(np.mean(e2e_times))
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    per_launch = {name: ms / max(cnt, 1) for name, (cnt, ms) in kt.items()}
    top = max(per_launch, key=per_launch.get)
    top_bytes = n * (JAM_DETECT_BYTES if top == "jam_stft_detect" else JAM_WIDEBAND_BYTES)
    achieved = top_bytes / (per_launch[top] / 1e3) / 1e9
    alg = n * (JAM_DETECT_BYTES + JAM_WIDEBAND_BYTES + JAM_COPY_BYTES)
    line = {
        "metric": "interference stage samples/s", "value": world * n / t_step, "unit": "samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (device-synthesised, seeded)",
        "config": {"workload": workload, "samples": n, "detections": [(d["type"], d["frequency_bin"]) for d in dets],
                   "parallelism": f"replicas x{world}", "l2": f"input {n * 8 / 1e6:.0f} MB > L2, restored before each step"},
        "e2e": {"value": world * n / t_e2e, "unit": "samples/s", "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8,
                "ms_per_step": t_e2e * 1e3},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": top_bytes,
                     "kernel_ms": {k: v for k, v in per_launch.items()},
                     "step_hbm_gbs": alg / t_step / 1e9,
                     "peak_source": "hbm_gbs of MEASURED_PEAKS.json"},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = jamming_cpu_baseline(h_pristine)
    return line


# ------------------------------------------------------------- observables
OBS_CHANNELS = 256
OBS_EPOCHS = 60_000  # one minute of 1 ms epochs: two LNAV frames for ephemeris decoding
# algorithmic bytes per channel-epoch: the bank's 88-byte output record read
# once (the fields Observable needs touch each of its 32-byte sectors) and
# the 32-byte observable written once
OBS_BYTES = 88 + 32
OBS_FS = 20e6
OBS_CAP = 8192  # candidate epochs kept per channel (random LNAV data give ~5,000 a minute)


def observables_outputs(dev):
    """Tracking-bank outputs of 256 channels x 60,000 epochs synthesised on
    the device from a fixed seed: prompt I/Q noise plus +-1 navigation
    symbols, carrier frequency near 2 kHz, loop errors, code phases.  Returns
    the raw (n_epochs, n_channels, 22) float32 buffer (88-byte records)."""
    import torch
    gen = torch.Generator(device=f"cuda:{dev}")
    gen.manual_seed(7)
    n_ep, n_ch = OBS_EPOCHS, OBS_CHANNELS
    rec = torch.zeros((n_ep, n_ch, 22), dtype=torch.float32, device=f"cuda:{dev}")
    rec[:, :, :10] = torch.randn((n_ep, n_ch, 10), generator=gen, device=f"cuda:{dev}") * 40
    bits = torch.randint(0, 2, (n_ep // 20 + 1, n_ch), generator=gen, device=f"cuda:{dev}").float() * 2 - 1
    rec[:, :, 4] += 300 * bits.repeat_interleave(20, dim=0)[:n_ep]
    d = rec.view(torch.float64)  # (n_ep, n_ch, 11): taps occupy 0..4
    d[:, :, 5] = 2000.0 + torch.randn((n_ep, n_ch), generator=gen, device=f"cuda:{dev}", dtype=torch.float64)
    d[:, :, 6] = torch.rand((n_ep, n_ch), generator=gen, device=f"cuda:{dev}", dtype=torch.float64) * 2 * np.pi
    d[:, :, 7] = 5000.0 + torch.rand((1, n_ch), generator=gen, device=f"cuda:{dev}", dtype=torch.float64) * 1000
    d[:, :, 8] = 1.023e6
    d[:, :, 9] = torch.randn((n_ep, n_ch), generator=gen, device=f"cuda:{dev}", dtype=torch.float64) * 0.02
    return rec


def observables_rows_host(n_ch):
    """The device synthesis's distribution for `n_ch` channels, drawn on the
    host with numpy (the reference arm needs no GPU): TRACK_DTYPE rows."""
    from ugsdr_gb300.api import TRACK_DTYPE
    rng = np.random.default_rng(7)
    n_ep = OBS_EPOCHS
    rows = np.zeros((n_ep, n_ch), TRACK_DTYPE)
    taps = rng.normal(0, 40, (n_ep, n_ch, 5, 2)).astype(np.float32)
    taps[:, :, 2, 0] += 300 * np.repeat(rng.choice([-1, 1], (n_ep // 20 + 1, n_ch)), 20, axis=0)[:n_ep]
    rows["taps"] = taps
    rows["carrier_frequency"] = 2000.0 + rng.normal(0, 1, (n_ep, n_ch))
    rows["carrier_phase"] = rng.random((n_ep, n_ch)) * 2 * np.pi
    rows["code_phase"] = 5000.0 + rng.random((1, n_ch)) * 1000
    rows["code_frequency"] = 1.023e6
    rows["phase_error"] = rng.normal(0, 0.02, (n_ep, n_ch))
    return rows


def observables_channels():
    return [dict(fs=OBS_FS, intermediate_frequency=0.0, carrier_frequency=2000.0, carrier_phase=0.0,
                 preamble_position=100, range_correction_ms=68.0) for _ in range(OBS_CHANNELS)]


def observables_cpu_baseline(rows, channels=32):
    """Observable's arithmetic and the preamble search restated in the oracle
    (obs_oracle.cpp), one thread, on the first `channels` channels."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    t0 = time.perf_counter()
    for c in range(channels):
        pyoracle.observables(rows[:, c], OBS_FS, 0.0, 2000.0, 0.0, 100, 68.0)
        pyoracle.preamble_search(rows["taps"][:, c, 2, 0], pyoracle.NAV_GPS_LNAV, cap=rows.shape[0])
    dt = time.perf_counter() - t0
    units = channels * rows.shape[0]
    return {"value": units / dt, "unit": "channel-epochs/s", "cores": 1, "kind": "port",
            "sample": f"{channels} channels x {rows.shape[0]} epochs in {dt:.2f}s (oracle observables + "
                      "preamble search, one thread)"}


def run_observables(args, world, rank):
    """Tracking outputs -> observables: ugsdr_observables (pseudorange,
    pseudophase, Doppler, SNR) and ugsdr_preamble_search (GPS LNAV) over 256
    channels x 60,000 epochs per step, outputs resident on the device."""
    from ugsdr_gb300 import api
    if args.impl == "reference" and rank != 0:
        return None
    n_ep, n_ch = OBS_EPOCHS, OBS_CHANNELS
    units = n_ep * n_ch
    workload = (f"observables: Observable arithmetic + FindPreambleGps candidates, {n_ch} channels x {n_ep} "
                f"epochs of tracking outputs")
    if args.impl == "reference":
        rows = observables_rows_host(32)  # the channels the bounded sample times
        vals = [observables_cpu_baseline(rows) for _ in range(args.warmup + args.steps)][args.warmup:]
        v = float(np.mean([b["value"] for b in vals]))
        return {"metric": "observables channel-epochs/s", "value": v, "unit": "channel-epochs/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": units / v * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": {"workload": workload},
                "cpu_baseline": {k: vals[-1][k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": v, "unit": "channel-epochs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    import torch
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    rec = observables_outputs(dev)
    chans = observables_channels()
    msgs = [0] * n_ch
    ctx = api.Context(dev)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)  # the events below bracket the library's kernels
    torch.cuda.synchronize()
    obs = torch.empty((n_ep, n_ch, 4), dtype=torch.float64, device=f"cuda:{dev}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    h_rows = torch.empty(rec.shape, dtype=torch.float32, pin_memory=True)
    h_rows.copy_(rec)
    h_np = h_rows.numpy().view(api.TRACK_DTYPE).reshape(n_ep, n_ch)

    def timed(k, on_device):
        times, cands = [], None
        l0 = ctx.launch_count()
        for _ in range(k):
            flush.fill_(1)  # the 1.35 GB records exceed L2 anyway; this evicts the last step's tail
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            t0 = time.perf_counter()
            if on_device:
                api.observables(ctx, rec.data_ptr(), chans, shape=(n_ep, n_ch), out_ptr=obs.data_ptr())
                cands = api.preamble_search(ctx, rec.data_ptr(), msgs, cap=OBS_CAP, shape=(n_ep, n_ch), as_arrays=True)
            else:
                out = api.observables(ctx, h_np, chans)
                cands = api.preamble_search(ctx, h_np, msgs, cap=OBS_CAP, as_arrays=True)
                del out
            e.record()
            e.synchronize()
            times.append(max(s.elapsed_time(e) / 1e3, time.perf_counter() - t0))
        return times, (ctx.launch_count() - l0) / k, cands

    timed(args.warmup, True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ctx.enable_timing(True)
    ctx.reset_timing()
    with ClockSampler() as clk:
        times, launches, cands = timed(args.steps, True)
    kt = {name: ctx.kernel_time(name) for name in ("observables", "obs_preamble")}
    ctx.enable_timing(False)
    t_step = float(np.mean(times))
    if world > 1:
        t = torch.tensor([t_step], device=f"cuda:{dev}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
    e2e_times, _, _ = timed(max(2, args.steps // 2), False)
    t_e2e = float(np.mean(e2e_times))
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    per_launch = {name: ms / max(cnt, 1) for name, (cnt, ms) in kt.items()}
    top_bytes = units * OBS_BYTES
    achieved = top_bytes / (per_launch["observables"] / 1e3) / 1e9
    line = {
        "metric": "observables channel-epochs/s", "value": world * units / t_step, "unit": "channel-epochs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (device-synthesised tracking outputs, seeded)",
        "config": {"workload": workload, "channels": n_ch, "epochs": n_ep,
                   "candidates": int(cands[0].sum()), "parallelism": f"replicas x{world}",
                   "l2": f"records {units * 88 / 1e9:.2f} GB > L2; 256 MB written between steps"},
        "e2e": {"value": world * units / t_e2e, "unit": "channel-epochs/s", "h2d_bytes_per_step": 2 * units * 88,
                "d2h_bytes_per_step": units * 32 + 4 * n_ch * (1 + OBS_CAP),
                "ms_per_step": t_e2e * 1e3},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "observables (obs_sigma + obs_segsum + obs_emit)", "achieved": achieved,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": top_bytes, "kernel_ms": per_launch,
                     "peak_source": "hbm_gbs of MEASURED_PEAKS.json"},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = observables_cpu_baseline(h_np)
    return line


# ------------------------------------------------------------ CPU reference
CPU_FFT_NOTE = ("float transforms by the project's iterative Stockham FFT (oracle/fft64.hpp FftT<float>, plans "
                "cached per size); FFTW is absent here and on the GPU box, so the reference's FFTW build is not timed")


def cpu_sample(jobs, raw, fs, threads, codes_per_system=None):
    """One bounded sample of the workload on the host cores through the CPU
    restatement of the reference loop (oracle/, ProcessBpsk with per-code,
    per-Doppler re-mix and two transforms per block): for each system, as
    many codes as threads (or `codes_per_system`), 1 Doppler bin, the full K
    blocks (front-end jobs: 4 blocks, the front end timed on the same
    prefix).  Returns the seconds it took, the cells it searched and the
    per-cell rate scaled to the whole step."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    x = raw.astype(np.float32)
    x = (x[:, 0] + 1j * x[:, 1]).astype(np.complex64) if raw.ndim == 2 else x.astype(np.complex64)
    step_t, sample_t, sample_cells, desc = 0.0, 0.0, 0, []
    per_cell = {}
    t_start = time.perf_counter()
    for j in jobs:
        key = (j["system"], j["n"], j["k"])
        fs_in = j.get("fs_in", 0.0)
        ks = min(j["k"], 4) if fs_in else j["k"]
        t0 = time.perf_counter()
        if fs_in:
            need = int(np.ceil(j["n"] * ks * fs_in / fs)) + 2
            xx = pyoracle.table_mix(x[:need], fs_in, j["fe"]) if j["fe"] else x[:need]
            xx = pyoracle.resample(xx, int(fs), int(fs_in))[: j["n"] * ks]
        else:
            xx = pyoracle.table_mix(x[: j["n"] * j["k"]], fs, j["fe"]) if j["fe"] else x[: j["n"] * j["k"]]
        t_front = (time.perf_counter() - t0) * j["k"] / ks  # once per job, scaled to K
        step_t += t_front
        if key not in per_cell:
            ncodes = min(len(j["codes"]), codes_per_system or threads)
            codes = np.stack([oracle_code(pyoracle, j, c) for c in j["codes"][:ncodes]])
            t0 = time.perf_counter()
            pyoracle.fse_baseline(xx, j["n"], ks, codes, fs, 0.0, 1.0, threads=threads)
            dt = time.perf_counter() - t0
            per_cell[key] = dt / (ncodes * j["n"]) * j["k"] / ks
            sample_cells += ncodes * j["n"]
            desc.append(f"{j['system']}: {ncodes} codes x 1 Doppler x {j['n']} x {ks} blocks in {dt:.2f} s"
                        + (f" (scaled to {j['k']} blocks)" if ks != j["k"] else ""))
        step_t += per_cell[key] * job_cells(j)
    sample_t = time.perf_counter() - t_start
    cells = sum(job_cells(j) for j in jobs)
    return {"value": cells / step_t, "sample_seconds": sample_t, "sample_cells": sample_cells,
            "full_step_seconds_extrapolated": step_t, "sample": "; ".join(desc)}


def cpu_anchor_gps_4mhz(threads):
    """The full-size GPS L1 C/A 4 MHz search (32 PRN x 21 Doppler x 4000 x 10,
    int8), timed whole on the host cores: no extrapolation."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    jobs, raw = gps_4mhz_workload()
    j = jobs[0]
    x = raw.astype(np.float32)
    x = (x[:, 0] + 1j * x[:, 1]).astype(np.complex64)
    codes = np.stack([oracle_code(pyoracle, j, c) for c in j["codes"]])
    t0 = time.perf_counter()
    pyoracle.fse_baseline(x[: j["n"] * j["k"]], j["n"], j["k"], codes, j["fs"], 5000.0, j["step"], threads=threads)
    dt = time.perf_counter() - t0
    cells = job_cells(j)
    return {"workload": WORKLOAD_DESC["gps_l1_4mhz"], "seconds": dt, "cells": cells, "value": cells / dt,
            "unit": "cells/s", "cores": threads, "extrapolated": False}


def repo_libraries():
    """Shared objects of this repository mapped into this process."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return []
    return sorted({l.split()[-1] for l in maps if l.endswith(".so") and str(ROOT) in l})


def cpu_baseline(args, jobs, raw, fs):
    """The ours-arm line's cpu_baseline: one sample on all host threads."""
    threads = os.cpu_count() or 1
    b = cpu_sample(jobs, raw, fs, threads)
    return {"value": b["value"], "unit": "cells/s", "cores": threads, "kind": "port", "extrapolated": True,
            "sample": b["sample"] + f" ({b['sample_seconds']:.2f} s wall) -> per-cell time x cells of the full step; "
                      + CPU_FFT_NOTE,
            "ms_per_step_extrapolated": b["full_step_seconds_extrapolated"] * 1e3}


def run_reference(args, world, rank):
    """The reference path on the host cores: each step is one bounded sample
    of the workload (cpu_sample) on all host threads; `value` is the per-cell
    rate of the samples scaled to the workload's cells, `ms_per_step` the
    measured wall time of one sample step.  Also in the line: the same sample
    on one thread (the reference as written: par_unseq runs serially in
    libstdc++ without TBB) and the full-size 4 MHz search timed whole."""
    if rank != 0:
        return None
    jobs, raw = WORKLOADS[args.config]()
    fs = jobs[0].get("fs", FS)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(jobs, raw, fs, threads)
    vals = [cpu_sample(jobs, raw, fs, threads) for _ in range(args.steps)]
    v = float(np.median([b["value"] for b in vals]))
    ms = float(np.median([b["sample_seconds"] for b in vals])) * 1e3
    one = cpu_sample(jobs, raw, fs, 1, codes_per_system=1)
    cells = sum(job_cells(j) for j in jobs)
    b = vals[-1]
    return {
        "metric": "acq cells/s (PRN x Doppler x code-phase)", "value": v, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD_DESC.get(args.config, args.config), "cells_per_step": cells,
                   "step": "one bounded sample of the workload (1 Doppler bin per code, see cpu_baseline.sample); "
                           "value = its per-cell rate x the workload's cells (extrapolated)",
                   "sample_cells_per_step": b["sample_cells"]},
        "cpu_baseline": {"value": v, "unit": "cells/s", "cores": threads, "kind": "port", "extrapolated": True,
                         "sample": b["sample"] + "; " + CPU_FFT_NOTE,
                         "ms_per_full_step_extrapolated": cells / v * 1e3},
        "single_thread": {"value": one["value"], "unit": "cells/s", "cores": 1, "extrapolated": True,
                          "sample_seconds": one["sample_seconds"], "sample": one["sample"]},
        "anchor_full_search": cpu_anchor_gps_4mhz(threads),
        "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "libraries_loaded": [str(Path(x).relative_to(ROOT)) for x in repo_libraries()],
    }


# ------------------------------------------------------------- DFT stage
DFT25_TRANSFORMS = 1 << 22  # 1.05e8 points, 839 MB each way (> L2)


def run_dft25(args, world, rank):
    """The radix-25 DFT stage two ways (ugsdr_dft25_batch): the CUDA-core
    butterfly (the transforms' choice, `value`) and the tcgen05 3xTF32
    product (`tensor_cores`), each over 2^22 transforms of device data; the
    kernel times are the entry's CUDA events, best over the steps."""
    import ctypes as C

    import torch
    from ugsdr_gb300 import api

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ctx = api.Context(dev)
    n = DFT25_TRANSFORMS
    x = torch.randn(n * 50, device=f"cuda:{dev}")
    y = torch.empty_like(x)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    res = {}
    with ClockSampler() as clk:
        for method in (0, 1):
            times = []
            for step in range(args.warmup + args.steps):
                flush.zero_()
                ms = C.c_float()
                ctx._check(ctx.lib.ugsdr_dft25_batch(ctx.h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), n, method,
                                                     C.byref(ms)))
                if step >= args.warmup:
                    times.append(ms.value)
            res[method] = min(times)
    pts = n * 25
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    gbs = 16 * pts / (res[0] / 1e3) / 1e9  # 8 B read + 8 B written per point
    ctx.close()
    return {
        "metric": "25-point DFT stage points/s", "value": pts / (res[0] / 1e3), "unit": "points/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res[0], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (normal random complex input on the device)",
        "config": {"workload": f"{n} forward 25-point DFTs (the radix-25 butterfly of the four-step inverse), "
                               "device in / out, tiles of 128 transforms staged in shared memory",
                   "l2": "flushed between steps (256 MB write); data 839 MB each way > L2"},
        "e2e": None, "gpu_launches": 1,
        "roofline": {"bound": "hbm", "kernel": "dft25_cuda_kernel", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": gbs / hbm_peak, "traffic": None},
        "tensor_cores": {"kernel": "dft25_tc_kernel (tcgen05.mma kind::tf32, 3xTF32, M128 N64 K8 x 21 per tile)",
                         "value": pts / (res[1] / 1e3), "ms_per_step": res[1], "ratio_to_cuda_cores": res[0] / res[1]},
        "clocks": clk.summary(),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(WORKLOADS) + ["track", "jamming", "observables", "dft25"], default="multi")
    ap.add_argument("--track-seconds", type=float, default=10.0, help="capture length of --config track")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-served", action="store_true", help="skip the served section of the default line")
    ap.add_argument("--no-tune", action="store_true", help="keep the built-in tile rule (skip ugsdr_autotune)")
    ap.add_argument("--served", action="store_true", help="run the served request stream instead")
    ap.add_argument("--requests", type=int, default=24, help="requests in the served stream")
    ap.add_argument("--inflight", type=int, default=4, help="server slots for the served stream")
    ap.add_argument("--rate", type=float, default=2000.0, help="Poisson arrival rate of the served stream (req/s)")
    ap.add_argument("--policy", choices=["fifo", "response_ratio"], default="response_ratio",
                    help="server admission order for the served stream")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", 1))
    rank = int(os.environ.get("RANK", 0))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.served:
        print(json.dumps(run_served(args)), flush=True)
        return
    if args.config == "track":
        line = run_track(args, world, rank)
    elif args.config == "jamming":
        line = run_jamming(args, world, rank)
    elif args.config == "observables":
        line = run_observables(args, world, rank)
    elif args.config == "dft25":
        line = run_dft25(args, world, rank) if rank == 0 else None
    else:
        line = run_ours(args, world, rank) if args.impl == "ours" else run_reference(args, world, rank)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
