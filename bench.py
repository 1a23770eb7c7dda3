"""Benchmark of the Barger propagation hot path on GB300.

Default workload (the precision-study configuration): atmospheric propagation through a
59-shell synthetic Earth (equal-thickness shells, seeded monotone density 13.1 -> 2.6 g/cm^3
with a step at 3480 km), 2000 cos(zenith) x 2000 log-spaced energies (0.1-100 GeV), production
height 22 km, neutrino and antineutrino, nominal oscillation parameters, mixed-precision
kernels.  One step = both neutrino types over the full grid = 72e6 probabilities.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload atmos59|prem4|beam]

Prints one JSON line.  ``value`` is probabilities/s with inputs resident on the device
(CUDA events on the launching stream, max over ranks); ``e2e`` is the same metric through the
public API with host buffers (grid upload and full result download in the timed region);
``roofline`` reports the per-bin kernel against the live-measured FP32 FMA peak.
``--impl reference`` times the CPU oracle (C restatement of the reference's CPU
propagator, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import tempfile
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TYPES = 2  # neutrino + antineutrino per step
BATCH_SETS = 0  # --batch-sets: fewer parameter sets for the batched workloads (profiling)

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant kernel from one
# ncu capture each, summarised under profiles/: (bytes, the captured launch's result bytes,
# summary).  A launch of another size is scaled by its result bytes, since traffic is the
# output stream plus a small table/descriptor read that grows with it.
NCU_TRAFFIC = {
    ("atmos59", "mixed"): (5.914112e6 + 85.716992e6, 144.0e6,
                           "profiles/atmos_mixed_kernel_59shells_2000x2000.md"),
    # the table launch and the bin launch of one run
    ("batch_atmos", "mixed"): (0.435456e6 + 0.033280e6 + 83.864320e6 + 902.968832e6, 912.332288e6,
                               "profiles/batch_kernel_prem12_48problems.md"),
    ("batch_beam", "mixed"): (107.312384e6 + 912.375040e6, 921.6e6,
                              "profiles/batch_kernel_beam_128problems.md"),
    ("atmos59", "fp64"): (9.935872e6 + 245.010688e6, 288.0e6,
                          "profiles/atmos_f64_kernel_59shells_2000x2000.md"),
}


# The dominant kernel's measured pipe utilisation in the same captures: the fraction of the
# FMA (FP32) or FP64 pipe's peak the kernel keeps busy.  The canonical roofline fraction
# counts the reference formulation's flops, more than these kernels execute (it can exceed
# 1); this is the utilisation of what they do execute.
NCU_PIPE = {
    ("atmos59", "mixed"): ("sm__pipe_fma_cycles_active", 0.7233),
    ("batch_atmos", "mixed"): ("sm__pipe_fma_cycles_active", 0.6699),  # the bin launch
    ("batch_beam", "mixed"): ("sm__pipe_fma_cycles_active", 0.6852),
    ("atmos59", "fp64"): ("sm__pipe_fp64_cycles_active", 0.8926),
}


def ncu_pipe(workload, prec):
    """{metric: fraction} of the committed capture, or {} if there is none."""
    t = NCU_PIPE.get((workload, prec))
    return {"ncu_pipe_active": {t[0]: t[1], "source": NCU_TRAFFIC[(workload, prec)][2]}} if t else {}


def ncu_traffic(workload, prec, result_bytes):
    """(traffic bytes of one launch of result_bytes, note) from the committed capture."""
    t = NCU_TRAFFIC.get((workload, prec))
    if t is None:
        return None, None
    note = f"ncu dram read+write of a captured launch with {t[1]:.4g} result bytes ({t[2]})"
    if abs(result_bytes - t[1]) > 1:
        note += ", scaled by result bytes"
    return round(t[0] * result_bytes / t[1]), note


def f_bin(M):
    """Canonical algorithmic flops of one (cos, E) bin crossing M shells: eigen-solve 40 +
    phase 7 + 3-term transition matrix 183 per distinct segment (M+1), 216 per layer product
    (2M-1 of them), 27 for the nine |A|^2."""
    M = np.asarray(M, dtype=np.float64)
    return 27.0 + 230.0 * (M + 1) + 216.0 * np.maximum(2 * M - 1, 0)


def max_over_ranks(x, world, device):
    """x maximised over the ranks of the process group (the step time of the slowest rank)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def rank_seed(seed, rank):
    """Seed of a rank's shard: rank 0 keeps the configuration's own sets, the others draw
    independent ones (weak scaling: every rank propagates different parameter sets)."""
    return seed + 7919 * rank


def rank_parameter_set(rank, world):
    """The oscillation parameters a rank propagates in the single-grid workloads."""
    from cudaprob3_gb300 import earth
    return earth.NOMINAL if rank == 0 else earth.gaussian_sets(world, seed=77)[rank]


def workload(name, rank=0):
    from cudaprob3_gb300 import earth
    if name == "atmos59":
        r, rho, ye = earth.synthetic_shells(59)
        return dict(kind="atmos", model=(r, rho, ye), cz=earth.cosine_grid(2000),
                    en=earth.log_energy_grid(2000), h=22.0,
                    desc="atmospheric, 59 equal shells (seeded monotone profile), 2000 cos x "
                         "2000 log-E (0.1-100 GeV), h=22 km, nu+nubar")
    if name == "prem4":
        return dict(kind="atmos", model=earth.PREM_4LAYER, cz=earth.cosine_grid(400),
                    en=earth.log_energy_grid(400), h=22.0,
                    desc="atmospheric, PREM 4-layer, 400 cos x 400 log-E (0.1-100 GeV), "
                         "h=22 km, nu+nubar")
    if name == "beam":
        return dict(kind="beam", en=earth.lin_energy_grid(100000), rho=2.6, L=1300.0,
                    desc="beam, rho=2.6 g/cm^3, L=1300 km, 1e5 E (0.1-10 GeV), nu+nubar")
    if name == "batch_atmos":
        n = BATCH_SETS or 256
        sets = earth.gaussian_sets(n, seed=rank_seed(2024, rank))
        grids = earth.uneven_grids(n, seed=rank_seed(2025, rank))
        return dict(kind="batch", model=earth.PREM_12LAYER, h=22.0, sets=sets, grids=grids,
                    beam=None,
                    desc="batched atmospheric: 256 Gaussian parameter sets (half inverted "
                         "ordering), own grids n_cos U[100,1000] x n_E U[100,2000], PREM "
                         "12-layer, h=22 km, nu+nubar (512 problems), one CUDA-graph run (table "
                         "launch + persistent bin launch)")
    if name == "batch_beam":
        sets = earth.gaussian_sets(BATCH_SETS or 4096, seed=rank_seed(2026, rank))
        return dict(kind="batch", model=None, h=None, sets=sets, grids=None,
                    beam=dict(en=earth.lin_energy_grid(100000), rho=2.6, L=[295.0, 1300.0]),
                    desc="batched beam: 4096 Gaussian parameter sets (half inverted ordering), "
                         "1e5 E (0.1-10 GeV), rho=2.6, L=295 and 1300 km, nu+nubar "
                         "(8192 problems), one persistent launch")
    if name == "serve":
        return dict(kind="serve", desc="serving: 64 closed-loop chains, requests of atm 200^2, "
                                       "500^2, 2000^2 and beam 1e4, 1e5 bins (PREM 4-layer)")
    raise SystemExit(f"unknown workload {name}")


def problem_bins(w):
    """Bins of each problem of a batched workload (nu and nubar share their grid)."""
    if w["model"] is not None:
        return [nc * ne for nc, ne in w["grids"]]
    return [len(w["beam"]["en"]) * len(w["beam"]["L"])] * len(w["sets"])


def build_batch(w):
    from cudaprob3_gb300 import earth
    from cudaprob3_gb300.batch import Batch
    b = Batch(0)
    flops = 0.0
    nbins = 0
    params = []  # (problem id, parameter set, antineutrino)
    if w["model"] is not None:
        b.set_earth(*w["model"], w["h"])
        r = np.asarray(w["model"][0], dtype=np.float64)
        rd = np.sort(r)[::-1]
        lim = -np.sqrt(1 - rd ** 2 / 6371.0 ** 2)
        lim[0] = 0.0
        for m, (nc, ne) in zip(w["sets"], w["grids"]):
            cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
            M = (cz[:, None] < lim[None, :]).sum(axis=1)
            for anti in (False, True):
                pid = b.add_atmos(cz, en)
                b.set_params(pid, m, anti)
                params.append((pid, m, anti))
                flops += float(f_bin(M).sum()) * ne
                nbins += nc * ne
    else:
        bw = w["beam"]
        for m in w["sets"]:
            for anti in (False, True):
                pid = b.add_beam(bw["en"], bw["rho"], bw["L"])
                b.set_params(pid, m, anti)
                params.append((pid, m, anti))
                flops += float(f_bin(0)) * len(bw["en"]) * len(bw["L"])
                nbins += len(bw["en"]) * len(bw["L"])
    b.commit()
    return b, flops, nbins, params


def run_batch(args, w, rank, world):
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    b, flops, nbins, params = build_batch(w)
    t0 = time.perf_counter()
    b.tune(use_cache=True)
    tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.run()
    b.synchronize()
    ms = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            b.run()
            ms.append(b.synchronize())
    t_ms = max_over_ranks(float(np.mean(ms)), world, "cuda")
    probs = 9 * nbins

    # end to end through the public API: every step uploads each problem's parameters
    # (cp3_batch_set_params), runs, and downloads every result into page-locked host memory
    # (one reused buffer of the largest result: the bytes cross the link all the same)
    largest = max(9 * npb for npb in problem_bins(w))
    host = torch.empty(largest, dtype=torch.float32, pin_memory=True)

    def e2e_step():
        for pid, m, anti in params:
            b.set_params(pid, m, anti)
        b.run()
        for pid, _, _ in params:
            b.copy_result_async(pid, host.data_ptr())
        b.synchronize_stream()

    e2e_steps = min(args.steps, 3)
    e2e_step()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / e2e_steps, world, "cuda")
    peaks = fma_peaks(dev)
    achieved = flops / (t_ms * 1e-3) / 1e12
    info = b.info()
    # the split applies where there are eigen tables to build (atmospheric problems)
    launches = 2 if (b.split_tables() and w["model"] is not None) else 1
    line = {
        "metric": "oscillation probabilities/s (mixed precision, max err <= 1e-5 vs FP64 oracle)",
        "value": world * probs / (t_ms * 1e-3), "unit": "probabilities/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded parameter sets and grids)",
        "config": {"workload": args.workload, "description": w["desc"], "precision": "mixed",
                   "probabilities_per_step": probs, "problems": info["problems"],
                   "tiles": info["tiles"], "result_bytes": info["result_bytes"],
                   "tile_shape": b.shape(), "split_tables": b.split_tables(), "autotune_s": round(tune_s, 2),
                   "l2": f"per-run output {info['result_bytes'] / 1e9:.1f} GB exceeds L2"},
        "e2e": {"value": world * probs / (e2e_ms * 1e-3), "unit": "probabilities/s",
                "h2d_bytes_per_step": len(params) * b.parameter_bytes(),
                "d2h_bytes_per_step": info["result_bytes"], "ms_per_step": e2e_ms,
                "steps": e2e_steps},
        "gpu_launches": args.steps * launches,
        "roofline": {"bound": "fp32", "achieved": round(achieved, 3),
                     "peak": round(peaks["fp32"], 3), "unit": "TFLOP/s",
                     "frac": round(achieved / peaks["fp32"], 4),
                     "traffic": ncu_traffic(args.workload, "mixed", info["result_bytes"])[0],
                     "traffic_note": ncu_traffic(args.workload, "mixed", info["result_bytes"])[1],
                     "kernel": "batch_kernel (%s per step)" % (
                         "a table launch and a bin launch" if launches == 2 else "one persistent launch"),
                     "flops_per_launch": flops,
                     "hbm_gbs_output": round(info["result_bytes"] / (t_ms * 1e-3) / 1e9, 1),
                     **ncu_pipe(args.workload, "mixed")},
        "peaks_tflops": peaks,
    }
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        line["roofline"]["hbm_frac_of_measured"] = round(line["roofline"]["hbm_gbs_output"] / mp["hbm_gbs"], 4)
    except (OSError, KeyError, ValueError):
        pass
    if rank == 0:
        line["max_abs_err_vs_oracle"] = check_batch_against_oracle(w, b)
    line["clocks"] = clk.summary()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, seconds=args.cpu_seconds)
    return line


def run_batch_fp64(args, w, rank, world):
    """The batched workload through the plain FP64 kernels: one FP64 handle per problem
    (created before the timed region), one launch each on one stream, timed with CUDA events
    around the whole loop.  This is the like-for-like baseline of the mixed batch."""
    import torch
    from cudaprob3_gb300 import earth
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    props, flops, nbins = [], 0.0, 0
    if w["model"] is not None:
        r = np.asarray(w["model"][0], dtype=np.float64)
        lim = -np.sqrt(1 - np.sort(r)[::-1] ** 2 / 6371.0 ** 2)
        lim[0] = 0.0
        for m, (nc, ne) in zip(w["sets"], w["grids"]):
            cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
            M = (cz[:, None] < lim[None, :]).sum(axis=1)
            for knu in (1, -1):
                p = make_propagator(dict(kind="atmos", cz=cz, en=en, model=w["model"], h=w["h"]),
                                    "fp64")
                set_params(p, m, knu)
                props.append((p, 0 if knu == 1 else 1))
                flops += float(f_bin(M).sum()) * ne
                nbins += nc * ne
    else:
        # the first 512 sets (2048 handles, 15 GB of FP64 results): the rate does not depend
        # on how many sets run, and the full 8192 x 2 handles would hold 118 GB
        bw = w["beam"]
        for m in w["sets"][:512]:
            for knu in (1, -1):
                for L in bw["L"]:
                    p = make_propagator(dict(kind="beam", en=bw["en"], rho=bw["rho"], L=L), "fp64")
                    set_params(p, m, knu)
                    props.append((p, 0 if knu == 1 else 1))
                    flops += float(f_bin(0)) * len(bw["en"])
                    nbins += len(bw["en"])
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    def step():
        for p, t in props:
            p.calculate_async(t, sp)

    for _ in range(max(1, min(args.warmup, 2))):
        step()
    stream.synchronize()
    steps = max(1, min(args.steps, 3))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev) as clk:
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        e1.synchronize()
    t_ms = max_over_ranks(e0.elapsed_time(e1) / steps, world, "cuda")
    probs = 9 * nbins
    peaks = fma_peaks(dev)
    return {
        "metric": "oscillation probabilities/s, plain FP64 kernels (reference tolerance 1e-12)",
        "value": world * probs / (t_ms * 1e-3), "unit": "probabilities/s", "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": t_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded parameter sets and grids)",
        "config": {"workload": args.workload, "description": w["desc"], "precision": "fp64",
                   "probabilities_per_step": probs, "problems": len(props),
                   "launches": "one FP64 handle per problem, launched back to back on one stream",
                   "l2": "per-run output exceeds L2"},
        "gpu_launches": steps * len(props) * (2 if w["model"] is not None else 1),
        "roofline": {"bound": "fp64", "achieved": round(flops / (t_ms * 1e-3) / 1e12, 3),
                     "peak": round(peaks["fp64"], 3), "unit": "TFLOP/s",
                     "frac": round(flops / (t_ms * 1e-3) / 1e12 / peaks["fp64"], 4),
                     "traffic": None, "flops_per_launch": flops},
        "peaks_tflops": peaks,
        "clocks": clk.summary(),
    }


def check_batch_against_oracle(w, b, n_check=4):
    """A few problems of the timed batch against the CPU oracle."""
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix, Oracle
    orc = Oracle()
    errs = []
    for i in range(n_check):
        k = (i * 37) % len(w["sets"])
        m = w["sets"][k]
        for anti in (False, True):
            pid = 2 * k + int(anti)
            om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, -1 if anti else 1)
            got = b.result(pid)
            if w["model"] is not None:
                nc, ne = w["grids"][k]
                cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
                rows = np.arange(0, nc, max(1, nc // 40))
                ref = orc.atmos(om, anti, cz[rows], en, *w["model"], w["h"], nthreads=os.cpu_count() or 1)
                errs.append(float(np.abs(np.transpose(got, (1, 2, 0))[rows] - ref).max()))
            else:
                bw = w["beam"]
                for j, L in enumerate(bw["L"]):
                    ref = orc.beam(om, anti, bw["en"], bw["rho"], L, nthreads=os.cpu_count() or 1)
                    errs.append(float(np.abs(got[j].T - ref).max()))
    return max(errs)


def shells_crossed(w):
    from cudaprob3_gb300 import earth  # noqa: F401
    r = np.asarray(w["model"][0], dtype=np.float64)
    rd = np.sort(r)[::-1]
    lim = -np.sqrt(1 - rd ** 2 / 6371.0 ** 2)
    lim[0] = 0.0
    return (w["cz"][:, None] < lim[None, :]).sum(axis=1)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        # raw samples: $CP3_CLOCKS_DIR if set (kept), else a temporary directory
        d = os.environ.get("CP3_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, f"clocks_gpu{gpu_index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path).read().splitlines()[1:]:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax = float(parts[2].split()[0])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def fma_peaks(device):
    from cudaprob3_gb300 import build
    L = C.CDLL(build.PEAKS_LIB)
    L.cp3peaks_fma_tflops.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
    out = {}
    for name, mode, iters in (("fp32_scalar", 0, 8192), ("fp32_paired", 2, 4096), ("fp64", 1, 512)):
        t, ms = C.c_double(), C.c_double()
        rc = L.cp3peaks_fma_tflops(mode, device, iters, C.byref(t), C.byref(ms))
        out[name] = t.value if rc == 0 else None
    # The FP32 roofline is the faster of scalar and paired (two FMAs per instruction) FMA.
    fp32 = [v for v in (out["fp32_scalar"], out["fp32_paired"]) if v]
    out["fp32"] = max(fp32) if fp32 else None
    return out


def make_propagator(w, prec):
    from cudaprob3_gb300 import AtmosCudaPropagatorSingle, BeamCudaPropagatorSingle
    if w["kind"] == "atmos":
        p = AtmosCudaPropagatorSingle(0, len(w["cz"]), len(w["en"]), precision=prec)
        p.setEnergyList(w["en"])
        p.setCosineList(w["cz"])
        p.setDensity(*w["model"])
        p.setProductionHeight(w["h"])
    else:
        p = BeamCudaPropagatorSingle(0, len(w["en"]), 1, precision=prec)
        p.setEnergyList(w["en"])
        p.setDensity(w["rho"])
        p.setPathLength(w["L"])
    return p


def set_params(p, m, knu):
    p.setMNSMatrix(m.theta12, m.theta13, m.theta23, m.dcp, knu)
    p.setNeutrinoMasses(m.dm12sq, m.dm23sq)


def run_serve(args, rank, world):
    """Serving workload: 64 closed-loop chains (each waits for its result, then thinks for an
    exponential time and submits again) over request sizes {atm 200^2, 500^2, 2000^2; beam
    1e4, 1e5}; the think time is swept down to zero (saturation)."""
    import threading
    from cudaprob3_gb300 import earth
    from cudaprob3_gb300.serve import Server
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    srv = Server(dev, pool_bytes=16 << 30, max_batch=256, max_bins_per_launch=8_000_000)
    srv.set_earth(*earth.PREM_4LAYER, 22.0)
    kinds = []
    for n in (200, 500, 2000):
        kinds.append((f"atm{n}x{n}", srv.add_atmos_grid(earth.cosine_grid(n), earth.log_energy_grid(n)), n * n))
    for n in (10000, 100000):
        kinds.append((f"beam{n}", srv.add_beam_grid(earth.lin_energy_grid(n), 2.6, [1300.0]), n))
    srv.start()
    sets = earth.gaussian_sets(512, seed=31)
    n_chains = 64
    # warm-up: every kind once
    for _, g, _ in kinds:
        rid = srv.submit(g, sets[0], False)
        srv.wait(rid)
        srv.release(rid)
    levels = []
    for think_ms in (args.serve_think or [20.0, 5.0, 1.0, 0.0]):
        records, lock = [], threading.Lock()
        t_end = time.perf_counter() + args.serve_seconds

        def chain(cid):
            rng = np.random.default_rng(1000 * cid + int(think_ms * 10))
            local = []
            while time.perf_counter() < t_end:
                if think_ms > 0:
                    time.sleep(rng.exponential(think_ms * 1e-3))
                k = int(rng.integers(len(kinds)))
                rid = srv.submit(kinds[k][1], sets[int(rng.integers(len(sets)))], bool(rng.integers(2)))
                srv.wait(rid, 60.0)
                local.append((k, srv.latency_ms(rid)))
                srv.release(rid)
            with lock:
                records.extend(local)

        st0 = srv.stats()
        t0 = time.perf_counter()
        th = [threading.Thread(target=chain, args=(c,)) for c in range(n_chains)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        wall = time.perf_counter() - t0
        st1 = srv.stats()
        lat = np.array([x[1] for x in records])
        kk = np.array([x[0] for x in records])
        probs = 9.0 * sum(kinds[k][2] for k in kk)
        lv = {"think_ms": think_ms, "requests": len(records),
              "requests_per_s": round(len(records) / wall, 1),
              "probabilities_per_s": probs / wall,
              "launches": st1["launches"] - st0["launches"],
              "p50_ms": round(float(np.percentile(lat, 50)), 3),
              "p99_ms": round(float(np.percentile(lat, 99)), 3)}
        for k, (name, _, _) in enumerate(kinds):
            sel = lat[kk == k]
            if len(sel):
                lv[name] = {"n": int(len(sel)), "p50_ms": round(float(np.percentile(sel, 50)), 3),
                            "p99_ms": round(float(np.percentile(sel, 99)), 3)}
        levels.append(lv)
    sat = levels[-1]
    srv.close()
    line = {
        "metric": "serving: probabilities/s at saturation (64 closed-loop chains), p50/p99 latency vs load",
        "value": sat["probabilities_per_s"], "unit": "probabilities/s", "n_gpus": world,
        "steps": len(levels), "warmup": 1, "ms_per_step": args.serve_seconds * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded parameter sets; PREM 4-layer, h=22 km; beam rho=2.6, L=1300 km)",
        "config": {"workload": "serve", "chains": n_chains,
                   "request_sizes": [k[0] for k in kinds], "pool_bytes": 16 << 30,
                   "max_bins_per_launch": 8_000_000, "scheduling": "smallest-first, 4 ms aging"},
        "latency_p99_atm500_at_saturation_ms": sat.get("atm500x500", {}).get("p99_ms"),
        "levels": levels,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(workload("serve"), seconds=args.cpu_seconds)
    return line


def run_ours(args, rank, world):
    import torch
    from cudaprob3_gb300 import earth

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if args.workload == "serve":
        return run_serve(args, rank, world)
    w = workload(args.workload, rank)
    if w["kind"] == "batch":
        if args.precision == "fp64":
            return run_batch_fp64(args, w, rank, world)
        return run_batch(args, w, rank, world)
    prec = args.precision
    # weak scaling: each rank propagates its own parameter set over the full grid
    m = rank_parameter_set(rank, world)
    props = []
    for knu in (1, -1):
        p = make_propagator(w, prec)
        set_params(p, m, knu)
        props.append(p)
    # A dedicated stream: kernels, events and the L2 flush are all ordered on it (the legacy
    # default stream's handle is 0, which the C ABI reads as "the handle's own stream").
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    assert sptr != 0
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # Neutrino and antineutrino on two streams forked from and joined back into `stream`, as
    # a caller with two handles would run them: one type's eigen-table kernel overlaps the
    # other's per-bin kernel.
    type_streams = [torch.cuda.Stream() for _ in props]

    def step():
        fork = torch.cuda.Event()
        fork.record(stream)
        done = []
        for t, p in enumerate(props):
            type_streams[t].wait_event(fork)
            p.calculate_async(t, type_streams[t].cuda_stream)
            e = torch.cuda.Event()
            e.record(type_streams[t])
            done.append(e)
        for e in done:
            stream.wait_event(e)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # numerical check of the timed configuration: nu and nubar against the CPU oracle on a
    # slice of cosine rows (the full grid would take the oracle minutes)
    max_err = check_against_oracle(w, props, m) if rank == 0 else None

    if w["kind"] == "atmos":
        nbins = len(w["cz"]) * len(w["en"])
        M = shells_crossed(w)
        flops_launch = float(f_bin(M).sum()) * len(w["en"])
    else:
        nbins = len(w["en"])
        flops_launch = float(f_bin(0)) * nbins
    probs_step = 9 * nbins * N_TYPES
    bytes_out_launch = 9 * nbins * (4 if prec == "mixed" else 8)

    # device-resident timed region: K steps, L2 flushed (untimed) between steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    bins_ms, eig_ms = [], []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        for k in range(args.steps):
            flush.add_(1.0)
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = max_over_ranks(float(np.mean(step_ms)), world, "cuda")
    if world > 1:
        torch.distributed.barrier()
    value = world * probs_step / (t_ms * 1e-3)

    # The roofline's kernel durations come from a second, serial pass (the two types one
    # after the other on one stream, L2 flushed before each): in the timed steps the types
    # overlap, so each kernel's wall time there includes the other's.
    for p in props:
        p.set_profiling(True)
    for k in range(max(3, args.steps)):
        for t, p in enumerate(props):
            flush.add_(1.0)
            p.calculate_async(t, sptr)
            a, b = p.kernel_times()
            eig_ms.append(a)
            bins_ms.append(b)
    for p in props:
        p.set_profiling(False)
    torch.cuda.synchronize()
    kernel_ms = float(np.mean(bins_ms))

    # end to end through the public API: grid H2D from pinned memory, compute, full D2H
    is_float = prec == "mixed"
    host_out = [torch.empty(bytes_out_launch // (4 if is_float else 8),
                            dtype=torch.float32 if is_float else torch.float64, pin_memory=True)
                for _ in props]
    en_pinned = torch.from_numpy(np.asarray(w["en"], dtype=np.float64)).pin_memory()
    cz_pinned = (torch.from_numpy(np.asarray(w["cz"], dtype=np.float64)).pin_memory()
                 if w["kind"] == "atmos" else None)

    # neutrino and antineutrino on their own streams, each computed in row pieces whose
    # downloads overlap the next piece's compute (cp3_calculate_to_host_async)
    e2e_streams = [torch.cuda.Stream() for _ in props]

    def e2e_step():
        for t, p in enumerate(props):
            p.setEnergyList(en_pinned.numpy())
            if cz_pinned is not None:
                p.setCosineList(cz_pinned.numpy())
            sp = e2e_streams[t].cuda_stream
            p.calculate_to_host_async(t, host_out[t].data_ptr(), 0, sp)
        for st in e2e_streams:
            st.synchronize()

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, world, "cuda")
    # bytes that cross the link: the energy lists; an unchanged cosine list is recognised
    # on the host (one memcmp) and not uploaded again
    h2d = len(w["en"]) * 8 * len(props)
    d2h = bytes_out_launch * len(props)

    peaks = fma_peaks(dev)
    achieved = flops_launch / (kernel_ms * 1e-3) / 1e12
    peak32 = peaks.get("fp32")
    roofline = {
        "bound": "fp32" if prec == "mixed" else "fp64",
        "achieved": round(achieved, 3),
        "peak": round(peak32 if prec == "mixed" else peaks.get("fp64"), 3),
        "unit": "TFLOP/s",
        "frac": round(achieved / (peak32 if prec == "mixed" else peaks.get("fp64")), 4),
        "traffic": ncu_traffic(args.workload, prec, bytes_out_launch)[0],
        "traffic_note": ncu_traffic(args.workload, prec, bytes_out_launch)[1],
        **ncu_pipe(args.workload, prec),
        "peak_source": "live FMA-chain microbenchmark in this run (cp3_peaks.cu); the pool's "
                       "measured HBM/bf16 peaks do not apply to scalar FP pipes",
        "kernel": "atmos_mixed_kernel" if (w["kind"] == "atmos" and prec == "mixed") else
                  ("atmos_f64_kernel" if w["kind"] == "atmos" else
                   ("beam_mixed_kernel" if prec == "mixed" else "beam_f64_kernel")),
        "kernel_ms": round(kernel_ms, 4),
        "eigen_table_ms": round(float(np.mean(eig_ms)), 4),
        "flops_per_launch": flops_launch,
        "hbm_gbs_output": round(bytes_out_launch / (kernel_ms * 1e-3) / 1e9, 1),
    }
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        roofline["hbm_frac_of_measured"] = round(roofline["hbm_gbs_output"] / mp["hbm_gbs"], 4)
    except (OSError, KeyError, ValueError):
        pass

    line = {
        "metric": "oscillation probabilities/s (mixed precision, max err <= 1e-5 vs FP64 oracle)",
        "value": value,
        "unit": "probabilities/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64" if prec == "mixed" else "f64",
        "data": "synthetic (seeded Earth model and parameters; no dataset involved)",
        "config": {"workload": args.workload, "description": w["desc"], "precision": prec,
                   "probabilities_per_step": probs_step,
                   "l2": "256 MB buffer written between timed steps (untimed); per-step output "
                         f"{d2h / 1e6:.0f} MB exceeds L2"},
        "e2e": {"value": world * probs_step / (e2e_ms * 1e-3), "unit": "probabilities/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "gpu_launches": args.steps * len(props) * (2 if w["kind"] == "atmos" else 1),
        "max_abs_err_vs_oracle": max_err,
        "roofline": roofline,
        "peaks_tflops": peaks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, seconds=args.cpu_seconds)
    line["clocks"] = clk.summary()
    return line


def check_against_oracle(w, props, m):
    from oracle.oracle import Mixing as OMix, Oracle
    orc = Oracle()
    errs = []
    for t, p in enumerate(props):
        got = p.probabilities()
        knu = 1 if t == 0 else -1
        mix = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu)
        if w["kind"] == "atmos":
            rows = np.arange(0, len(w["cz"]), max(1, len(w["cz"]) // 50))
            r, rho, ye = w["model"]
            ref = orc.atmos(mix, t == 1, w["cz"][rows], w["en"], r, rho, ye, w["h"],
                            nthreads=os.cpu_count() or 1)
            errs.append(float(np.abs(got[rows] - ref).max()))
        else:
            ref = orc.beam(mix, t == 1, w["en"], w["rho"], w["L"], nthreads=os.cpu_count() or 1)
            errs.append(float(np.abs(got - ref).max()))
    return max(errs)


def cpu_sample(w, seconds, orc=None, nthreads=1):
    """A bounded slice of the workload for the CPU, sized from a short probe run to take
    about ``seconds`` of wall time: every k-th cosine row (keeps the distribution of shells
    crossed) or a contiguous block of beam energies."""
    if w["kind"] == "atmos":
        stride = max(1, len(w["cz"]) // 8)
        if orc is not None:
            # a warm-up (library, thread pool), then a probe of four rows per thread
            stride = max(1, len(w["cz"]) // (4 * nthreads))
            probe = dict(w, cz=w["cz"][::stride])
            cpu_run(dict(probe, cz=probe["cz"][:nthreads]), orc, nthreads)
            t0 = time.perf_counter()
            cpu_run(probe, orc, nthreads)
            rows_per_s = len(probe["cz"]) / max(time.perf_counter() - t0, 1e-9)
            # enough rows that the dynamic schedule keeps every thread busy
            rows = max(8 * nthreads, min(len(w["cz"]), int(seconds * rows_per_s)))
            stride = max(1, len(w["cz"]) // rows)
        sub = w["cz"][::stride]
        if stride == 1:
            return dict(w, cz=sub), f"the whole grid ({len(sub)} x {len(w['en'])} bins), nu+nubar"
        return dict(w, cz=sub), f"every {stride}th cosine row ({len(sub)} x {len(w['en'])} bins), nu+nubar"
    n = len(w["en"])
    if orc is not None:
        probe = dict(w, en=w["en"][:20000])
        cpu_run(probe, orc, nthreads)  # warm-up
        t0 = time.perf_counter()
        cpu_run(probe, orc, nthreads)
        n = max(20000, min(n, int(seconds / max((time.perf_counter() - t0) / 20000, 1e-12))))
    return dict(w, en=w["en"][:n]), f"{n} energies, nu+nubar"


def cpu_run(w, orc, nthreads, m=None):
    """Probabilities/s of the C restatement on one single-grid workload, nu and nubar."""
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    m = m or earth.NOMINAL
    t0 = time.perf_counter()
    nbins = 0
    for anti, knu in ((False, 1), (True, -1)):
        mix = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu)
        if w["kind"] == "atmos":
            r, rho, ye = w["model"]
            orc.atmos(mix, anti, w["cz"], w["en"], r, rho, ye, w["h"], nthreads=nthreads)
            nbins += len(w["cz"]) * len(w["en"])
        else:
            for L in np.atleast_1d(w["L"]):
                orc.beam(mix, anti, w["en"], w["rho"], float(L), nthreads=nthreads)
                nbins += len(w["en"])
    return 9 * nbins / (time.perf_counter() - t0)


def cpu_jobs(w, seconds, orc, nthreads):
    """The CPU's share of a workload: (list of (single-grid workload, parameter set), text).
    Single grids are sliced by cpu_sample; batched workloads take their first parameter sets
    on their own grids, as many as fit about ``seconds``; serving takes 500 x 500 PREM-4
    requests (the size its latency target is quoted for)."""
    from cudaprob3_gb300 import earth
    if w["kind"] in ("atmos", "beam"):
        sw, desc = cpu_sample(w, seconds, orc, nthreads)
        return [(sw, None)], desc
    if w["kind"] == "serve":
        req = dict(kind="atmos", model=earth.PREM_4LAYER, cz=earth.cosine_grid(500),
                   en=earth.log_energy_grid(500), h=22.0)
        sets = earth.gaussian_sets(64, seed=4242)
        cands = [(req, m) for m in sets]
        what = "500 x 500 PREM-4 requests, one parameter set each"
    elif w["beam"] is not None:
        bw = w["beam"]
        cands = [(dict(kind="beam", en=bw["en"], rho=bw["rho"], L=bw["L"]), m) for m in w["sets"]]
        what = "beam problems (1e5 energies, both baselines), one parameter set each"
    else:
        cands = [(dict(kind="atmos", model=w["model"], cz=earth.cosine_grid(nc),
                       en=earth.log_energy_grid(ne), h=w["h"]), m)
                 for m, (nc, ne) in zip(w["sets"], w["grids"])]
        what = "atmospheric problems on their own grids, one parameter set each"
    jobs, t0 = [], time.perf_counter()
    for job in cands:  # the probe is the sample itself: stop once the budget is spent
        cpu_run(job[0], orc, nthreads, job[1])
        jobs.append(job)
        if time.perf_counter() - t0 >= seconds:
            break
    return jobs, f"the first {len(jobs)} {what}, nu+nubar"


def job_probs(w):
    """Probabilities of one single-grid job, nu and nubar."""
    if w["kind"] == "atmos":
        return 9 * N_TYPES * len(w["cz"]) * len(w["en"])
    return 9 * N_TYPES * len(w["en"]) * len(np.atleast_1d(w["L"]))


def run_jobs(jobs, orc, nthreads):
    """Probabilities/s over a list of jobs (one pass)."""
    t0 = time.perf_counter()
    for w, m in jobs:
        cpu_run(w, orc, nthreads, m)
    return sum(job_probs(w) for w, _ in jobs) / (time.perf_counter() - t0)


def cpu_baseline(w, seconds=2.0):
    from oracle.oracle import Oracle
    orc = Oracle(fast=True)
    cores = os.cpu_count() or 1
    jobs, desc = cpu_jobs(w, seconds, orc, cores)  # the sizing run also warms up
    rate = run_jobs(jobs, orc, cores)
    return {"value": rate, "unit": "probabilities/s", "cores": cores, "kind": "port",
            "sample": desc + "; C restatement of the reference CpuPropagator<double> "
                             "(OpenMP over cosines, -O3), all host threads"}


def run_reference(args):
    """The reference arm: the reference's CPU algorithm (C restatement) on the host cores."""
    from oracle.oracle import Oracle
    w = workload(args.workload)
    orc = Oracle(fast=True)
    cores = os.cpu_count() or 1
    jobs, desc = cpu_jobs(w, args.cpu_seconds, orc, cores)
    for _ in range(max(0, args.warmup - 1)):  # the sizing pass was the first warm-up
        run_jobs(jobs, orc, cores)
    rates = [run_jobs(jobs, orc, cores) for _ in range(args.steps)]
    value = float(np.median(rates))
    probs_step = sum(job_probs(j) for j, _ in jobs)
    return {
        "impl": "reference",
        "metric": "oscillation probabilities/s (mixed precision, max err <= 1e-5 vs FP64 oracle)",
        "value": value, "unit": "probabilities/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": probs_step / value * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": args.workload, "description": w["desc"],
                                        "sample": desc},
        "cpu_baseline": {"value": value, "unit": "probabilities/s", "cores": cores,
                         "kind": "port",
                         "sample": desc + "; reference CPU algorithm restated in C "
                                          "(oracle/cp3_oracle.c), the reference's own build "
                                          "needs its source tree, absent on this host"},
        "e2e": {"value": value, "unit": "probabilities/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="atmos59",
                    choices=["atmos59", "prem4", "beam", "batch_atmos", "batch_beam", "serve"])
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--serve-think", type=float, nargs="*", default=None,
                    help="mean think times (ms) of the chains, one load level each")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=2.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-sets", type=int, default=0,
                    help="parameter sets of the batched workloads (default: the configuration's)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    global BATCH_SETS
    BATCH_SETS = args.batch_sets

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    import __graft_entry__
    __graft_entry__.build()
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    line = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
