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
    ("atmos59", "mixed"): (5.910016e6 + 84.903680e6, 144.0e6,
                           "profiles/atmos_mixed_kernel_59shells_2000x2000.md"),
    # the table launch and the bin launch of one run
    ("batch_atmos", "mixed"): (0.431616e6 + 0.060672e6 + 205.593088e6 + 982.776320e6, 912.332288e6,
                               "profiles/batch_kernel_prem12_48problems.md"),
    ("batch_beam", "mixed"): (115.457024e6 + 911.392000e6, 921.6e6,
                              "profiles/batch_kernel_beam_128problems.md"),
    ("atmos59", "fp64"): (9.871104e6 + 244.749312e6, 288.0e6,
                          "profiles/atmos_f64_kernel_59shells_2000x2000.md"),
    # the 7.2 MB output is still in L2 when the captured launch ends
    ("beam", "fp64"): (0.865792e6, 7.2e6, "profiles/beam_f64_kernel_1e5energies.md"),
}


# The dominant kernel's measured pipe utilisation in the same captures: the fraction of the
# FMA (FP32) or FP64 pipe's peak the kernel keeps busy.  The canonical roofline fraction
# counts the reference formulation's flops, more than these kernels execute (it can exceed
# 1); this is the utilisation of what they do execute.
NCU_PIPE = {
    ("atmos59", "mixed"): ("sm__pipe_fma_cycles_active", 0.7099),
    ("batch_atmos", "mixed"): ("sm__pipe_fma_cycles_active", 0.6572),  # the bin launch
    ("batch_beam", "mixed"): ("sm__pipe_fma_cycles_active", 0.6007),
    ("atmos59", "fp64"): ("sm__pipe_fp64_cycles_active", 0.8930),
    ("beam", "fp64"): ("sm__pipe_fp64_cycles_active", 0.8518),
    ("batch_beam", "fp64"): ("sm__pipe_fp64_cycles_active", 0.8518),
}


def ncu_pipe(workload, prec):
    """{metric: fraction} of the committed capture, or {} if there is none."""
    t = NCU_PIPE.get((workload, prec))
    if not t:
        return {}
    src = NCU_TRAFFIC.get((workload, prec), NCU_TRAFFIC.get((workload.replace("batch_", ""), prec)))
    return {"ncu_pipe_active": {t[0]: t[1], "source": src[2] if src else None}}


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
        return dict(kind="serve", desc="serving: open-loop Poisson arrivals from 64 chains, "
                                       "requests of atm 200^2, 500^2, 2000^2 and beam 1e4, 1e5 "
                                       "bins (PREM 4-layer)")
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
    if args.shape:  # a fixed tile shape instead of the autotuner (profiling captures)
        b.set_shape(*args.shape)
    else:
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
    # (cp3_batch_set_params), runs, and downloads the whole result arena into page-locked
    # host memory.  Where the arena fits in a third of the host's memory (C2's 10.8 GB; C3's
    # 59 GB on a 199 GB host, pinned in ~5 s before the timed region),
    # cp3_batch_run_to_host runs the bins in windows of whole problems and downloads each
    # window while the next computes.  Otherwise the run is followed by copies of the arena
    # in 256 MB pieces into one reused buffer (cp3_batch_copy_results): the bytes cross the
    # link all the same.
    arena = b.info()["result_bytes"] // 4
    piece = 64 << 20  # floats
    try:
        host_mem = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError, AttributeError):
        host_mem = 0
    whole = 4 * arena <= host_mem // 3
    host = torch.empty(arena if whole else min(piece, arena), dtype=torch.float32, pin_memory=True)

    # Steps are queued back to back (set_params waits only until the previous step's
    # parameter upload has left the staging area); the timed region ends when the last
    # step's results are in host memory.
    def e2e_step(wait):
        for pid, m, anti in params:
            b.set_params(pid, m, anti)
        if whole:
            b.run_to_host(host.data_ptr())
        else:
            b.run()
            for first in range(0, arena, piece):
                b.copy_results_async(first, min(piece, arena - first), host.data_ptr())
        if wait:
            b.synchronize_stream()

    # Five trials of three steps each, the median trial reported: the device-to-host link
    # of this shared machine now and then slows a step by 4-18 ms (seen in the device-side
    # waits, not in host work), which would otherwise move a 3-step mean by up to a third.
    e2e_steps = min(args.steps, 3)
    e2e_step(True)
    trials, trials_sync = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step(False)
        b.synchronize_stream()
        trials.append((time.perf_counter() - t0) * 1e3 / e2e_steps)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step(True)
        trials_sync.append((time.perf_counter() - t0) * 1e3 / e2e_steps)
    e2e_ms = max_over_ranks(statistics.median(trials), world, "cuda")
    e2e_ms_sync = max_over_ranks(statistics.median(trials_sync), world, "cuda")
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
                "steps": e2e_steps, "steps_queued": "back to back",
                "trials_ms_per_step": [round(t, 3) for t in trials],
                "trials_ms_per_step_waiting_each_step": [round(t, 3) for t in trials_sync],
                "timing": "median of 5 trials of the steps",
                "download": ("cp3_batch_run_to_host: bins in windows of whole problems, each "
                             "window downloaded while the next computes" if whole else
                             "cp3_batch_run, then the arena in 256 MB copies into one reused "
                             "page-locked buffer"),
                "ms_per_step_waiting_each_step": e2e_ms_sync,
                "link": link_summary(info["result_bytes"], e2e_ms, d2h_link())},
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
        err, per, what = check_batch_against_oracle(w, b)
        line["max_abs_err_vs_oracle"] = err
        line["max_abs_err_per_channel"] = dict(per, channels="a*3+b = P(a->b): e_e, e_m, e_t, "
                                               "m_e, m_m, m_t, t_e, t_m, t_t", checked=what)
    line["clocks"] = clk.summary()
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        b.close()
        line["reference_fp64_gpu"] = reference_gpu_batch(w)
        if "value" in line["reference_fp64_gpu"]:
            line["mixed_over_reference_fp64_gpu"] = round(line["value"] / line["reference_fp64_gpu"]["value"], 1)
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
    props, flops, nbins, jobs = [], 0.0, 0, []
    if w["model"] is not None:
        r = np.asarray(w["model"][0], dtype=np.float64)
        lim = -np.sqrt(1 - np.sort(r)[::-1] ** 2 / 6371.0 ** 2)
        lim[0] = 0.0
        for m, (nc, ne) in zip(w["sets"], w["grids"]):
            cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
            M = (cz[:, None] < lim[None, :]).sum(axis=1)
            for knu in (1, -1):
                wk = dict(kind="atmos", cz=cz, en=en, model=w["model"], h=w["h"])
                p = make_propagator(wk, "fp64")
                set_params(p, m, knu)
                props.append((p, 0 if knu == 1 else 1))
                jobs.append((p, wk, m, knu))
                flops += float(f_bin(M).sum()) * ne
                nbins += nc * ne
    else:
        # the first 512 sets (2048 handles, 15 GB of FP64 results): the rate does not depend
        # on how many sets run, and the full 8192 x 2 handles would hold 118 GB
        bw = w["beam"]
        for m in w["sets"][:512]:
            for knu in (1, -1):
                for L in bw["L"]:
                    wk = dict(kind="beam", en=bw["en"], rho=bw["rho"], L=L)
                    p = make_propagator(wk, "fp64")
                    set_params(p, m, knu)
                    props.append((p, 0 if knu == 1 else 1))
                    jobs.append((p, wk, m, knu))
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
    # parity of the FP64 kernels on this batch: 8 handles spread over it, every bin
    from oracle.oracle import Mixing as OMix, Oracle
    orc, err = Oracle(), 0.0
    for p, wk, m, knu in [jobs[(i * (len(jobs) - 1)) // 7] for i in range(8)] if rank == 0 else []:
        om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu)
        if wk["kind"] == "atmos":
            ref = orc.atmos(om, knu < 0, wk["cz"], wk["en"], *wk["model"], wk["h"],
                            nthreads=os.cpu_count() or 1)
        else:
            ref = orc.beam(om, knu < 0, wk["en"], wk["rho"], wk["L"], nthreads=os.cpu_count() or 1)
        err = max(err, float(np.abs(p.probabilities() - ref).max()))
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
                     "traffic": None, "flops_per_launch": flops,
                     **ncu_pipe(args.workload, "fp64")},
        "peaks_tflops": peaks,
        "max_abs_err_vs_oracle": err if rank == 0 else None,
        "checked": "8 of the FP64 handles spread over the batch, every bin",
        "clocks": clk.summary(),
    }


def check_batch_against_oracle(w, b, n_check=12):
    """Problems of the timed batch against the CPU oracle: n_check parameter sets spread over
    the batch (both mass orderings), each with nu and nubar, every bin of their grids.
    Returns (max error, per-channel max errors for nu and nubar, what was checked)."""
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix, Oracle
    orc = Oracle()
    nt = os.cpu_count() or 1
    n_sets = len(w["sets"])
    picks = sorted({(i * (n_sets - 1)) // max(n_check - 1, 1) for i in range(n_check)})
    per = {"nu": np.zeros(9), "nubar": np.zeros(9)}
    for k in picks:
        m = w["sets"][k]
        for anti in (False, True):
            pid = 2 * k + int(anti)
            om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, -1 if anti else 1)
            got = b.result(pid)
            if w["model"] is not None:
                nc, ne = w["grids"][k]
                cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
                ref = orc.atmos(om, anti, cz, en, *w["model"], w["h"], nthreads=nt)
                err = np.abs(np.transpose(got, (1, 2, 0)) - ref).reshape(-1, 9).max(axis=0)
            else:
                bw = w["beam"]
                err = np.zeros(9)
                for j, L in enumerate(bw["L"]):
                    ref = orc.beam(om, anti, bw["en"], bw["rho"], L, nthreads=nt)
                    err = np.maximum(err, np.abs(got[j].T - ref).max(axis=0))
            key = "nubar" if anti else "nu"
            per[key] = np.maximum(per[key], err)
    what = (f"{len(picks)} of {n_sets} parameter sets spread over the batch (both orderings), "
            "nu and nubar, every bin of their grids")
    return float(max(per["nu"].max(), per["nubar"].max())), {k: v.tolist() for k, v in per.items()}, what


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


def d2h_link(nbytes=256 << 20, reps=5):
    """The device-to-host link's copy rate in GB/s, measured live: a page-locked copy of
    nbytes timed with CUDA events (median of reps).  On GB300 every route into host
    memory (copy engines on one or several streams, 2-D copies, SM stores of any width)
    measured the same rate, so this bounds any end-to-end step that downloads its results."""
    import torch
    src = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda").fill_(0.5)
    dst = torch.empty(nbytes // 4, dtype=torch.float32, pin_memory=True)
    s = torch.cuda.Stream()
    ms = []
    for _ in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s):
            e0.record(s)
            dst.copy_(src, non_blocking=True)
            e1.record(s)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return nbytes / (statistics.median(ms[1:]) * 1e-3) / 1e9


def link_summary(d2h_bytes, e2e_ms, gbs):
    """The e2e step's roofline: its bytes at the measured link rate, against its time."""
    return {"d2h_gbs_measured": round(gbs, 1),
            "d2h_gbs_achieved": round(d2h_bytes / (e2e_ms * 1e-3) / 1e9, 1),
            "frac_of_link": round(d2h_bytes / (e2e_ms * 1e-3) / 1e9 / gbs, 4)}


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


SERVE_P99_TARGET_MS = 2.0  # the serving latency target for 500 x 500 requests

SERVE_KINDS = (("atm200x200", "atmos", 200), ("atm500x500", "atmos", 500),
               ("atm2000x2000", "atmos", 2000), ("beam10000", "beam", 10000),
               ("beam100000", "beam", 100000))


def make_server(dev):
    """The serving configuration: PREM 4-layer at 22 km, the five request sizes registered,
    a 16 GB pool, up to 256 requests / 8e6 bins per launch."""
    from cudaprob3_gb300 import earth
    from cudaprob3_gb300.serve import Server
    srv = Server(dev, pool_bytes=16 << 30, max_batch=256, max_bins_per_launch=8_000_000)
    srv.set_earth(*earth.PREM_4LAYER, 22.0)
    kinds = []
    for name, kind, n in SERVE_KINDS:
        if kind == "atmos":
            g = srv.add_atmos_grid(earth.cosine_grid(n), earth.log_energy_grid(n))
            kinds.append((name, g, n * n))
        else:
            kinds.append((name, srv.add_beam_grid(earth.lin_energy_grid(n), 2.6, [1300.0]), n))
    srv.start()
    return srv, kinds


def serve_level(srv, kinds, sets, rate, seconds, n_chains=64, seed=0):
    """One offered load, open loop: each of n_chains chains is a Poisson process of
    rate/n_chains requests/s (together a Poisson process of `rate`).  Arrival times, request
    sizes, parameter sets and nu/nubar are drawn in advance from `seed`; one host thread
    submits each request at its arrival time, whatever is still outstanding, and collects
    completions through the server's completion queue.  A request's latency is its arrival
    time to the completion of its launch: the server's submit-to-completion time plus any
    delay of the submit behind its scheduled arrival."""
    rng = np.random.default_rng(seed)
    per_chain = rate / n_chains
    times = []
    for _ in range(n_chains):
        n = int(per_chain * seconds * 2) + 16
        t = np.cumsum(rng.exponential(1.0 / per_chain, size=n))
        times.append(t[t < seconds])
    times = np.sort(np.concatenate(times))
    n_req = len(times)
    kind = rng.integers(len(kinds), size=n_req)
    pset = rng.integers(len(sets), size=n_req)
    anti = rng.integers(2, size=n_req).astype(bool)
    srv.poll(0)  # start recording completions
    outstanding = {}
    lat = np.full(n_req, np.nan)
    t_done = np.full(n_req, np.inf)
    lag_max = 0.0
    i = done = 0
    st0 = srv.stats()
    deadline = seconds * 4 + 30.0
    t0 = time.perf_counter()
    now = 0.0
    while done < n_req and now < deadline:
        now = time.perf_counter() - t0
        while i < n_req and times[i] <= now:
            rid = srv.submit(kinds[kind[i]][1], sets[pset[i]], bool(anti[i]))
            lag = time.perf_counter() - t0 - times[i]
            lag_max = max(lag_max, lag)
            outstanding[rid] = (i, lag)
            i += 1
        wait = 0.05 if i >= n_req else max(0.0, min(times[i] - (time.perf_counter() - t0), 0.001))
        for rid in srv.poll(4096, wait):
            k, lag = outstanding.pop(rid)
            lat[k] = srv.latency_ms(rid) + lag * 1e3
            t_done[k] = time.perf_counter() - t0
            srv.release(rid)
            done += 1
    wall = time.perf_counter() - t0
    st1 = srv.stats()
    ok = ~np.isnan(lat)
    probs = 9.0 * sum(kinds[k][2] for k in kind[ok])
    # achieved: completions inside the arrival window over the window (an overloaded server
    # falls behind there; the backlog it clears afterwards does not count)
    lv = {"offered_req_per_s": round(rate, 1), "requests": int(n_req), "completed": int(ok.sum()),
          "achieved_req_per_s": round(float((t_done <= seconds).sum()) / seconds, 1),
          "probabilities_per_s": probs / wall, "launches": st1["launches"] - st0["launches"],
          "p50_ms": round(float(np.percentile(lat[ok], 50)), 3) if ok.any() else None,
          "p99_ms": round(float(np.percentile(lat[ok], 99)), 3) if ok.any() else None,
          "max_submit_lag_ms": round(lag_max * 1e3, 3), "seconds": round(wall, 3)}
    for k, (name, _, _) in enumerate(kinds):
        sel = lat[(kind == k) & ok]
        if len(sel):
            lv[name] = {"n": int(len(sel)), "p50_ms": round(float(np.percentile(sel, 50)), 3),
                        "p99_ms": round(float(np.percentile(sel, 99)), 3)}
    return lv


def serve_capacity(srv, kinds, sets, n=4000, seed=99):
    """Requests/s the server completes with a deep queue: n requests of the serving mix
    submitted at once, timed to the last completion.  It is the scale of the offered loads
    swept, not the knee: the sweep finds that."""
    rng = np.random.default_rng(seed)
    srv.poll(0)
    t0 = time.perf_counter()
    ids = [srv.submit(kinds[int(rng.integers(len(kinds)))][1], sets[int(rng.integers(len(sets)))],
                      bool(rng.integers(2))) for _ in range(n)]
    left = set(ids)
    while left and time.perf_counter() - t0 < 60.0:
        for rid in srv.poll(4096, 0.05):
            left.discard(rid)
            srv.release(rid)
    return n / (time.perf_counter() - t0)


def serve_sweep(dev, fractions, seconds, gpu_index):
    """Latency against offered load: the server's capacity from a deep-queue burst, then one
    open-loop level per fraction of it, each with its own clock record.  The knee is the
    highest offered load the server sustains: every request completed, the completions
    inside the arrival window at least 97 % of the arrivals, and the median latency within
    twice that of the lightest load (waiting in the queue does not dominate)."""
    from cudaprob3_gb300 import earth
    srv, kinds = make_server(dev)
    sets = earth.gaussian_sets(512, seed=31)
    for name, g, _ in kinds:  # warm-up: every size once
        rid = srv.submit(g, sets[0], False)
        srv.wait(rid, 60.0)
        srv.release(rid)
    serve_capacity(srv, kinds, sets, n=300)  # warm-up of the burst path
    # the median of three bursts: the offered loads are placed at fractions of it, and one
    # burst on a briefly busy host (seen once: 39k against 44k requests/s) would shift them all
    bursts = [serve_capacity(srv, kinds, sets, seed=99 + k) for k in range(3)]
    cap = statistics.median(bursts)
    levels = []
    for f in fractions:
        with Clocks(gpu_index) as clk:
            lv = serve_level(srv, kinds, sets, f * cap, seconds, seed=int(f * 1000))
        lv["fraction_of_capacity"] = f
        lv["clocks"] = clk.summary()
        levels.append(lv)
    srv.close()
    return cap, levels, serve_knee(levels, seconds), kinds, bursts


def serve_knee(levels, seconds):
    """The highest offered load sustained (see serve_sweep), or None."""
    p50s = [lv["p50_ms"] for lv in levels if lv["p50_ms"] is not None]
    if not p50s:
        return None
    p50_light = min(p50s)
    sustained = [lv for lv in levels
                 if lv["completed"] == lv["requests"]
                 and lv["achieved_req_per_s"] * seconds >= 0.97 * lv["requests"]
                 and lv["p50_ms"] <= 2.0 * p50_light]
    return max(sustained, key=lambda lv: lv["offered_req_per_s"]) if sustained else None


def serve_summary(cap, knee, kinds, levels=()):
    """The serving object of a bench line: the knee's offered load and latencies, and the
    level of the highest throughput (past the knee the queue grows for as long as the
    arrivals last, so latencies there measure the level's length as much as the server)."""
    top = max(levels, key=lambda lv: lv["achieved_req_per_s"]) if levels else None
    sat = None if top is None else {
        "offered_req_per_s": top["offered_req_per_s"], "achieved_req_per_s": top["achieved_req_per_s"],
        "probabilities_per_s": top["probabilities_per_s"], "p50_ms": top["p50_ms"],
        "p99_ms": top["p99_ms"], "atm500x500": top.get("atm500x500")}
    # the highest load at which 500 x 500 requests keep the 2 ms p99 target (every request
    # completed, the server keeping up)
    ok = [lv for lv in levels if lv.get("atm500x500") and lv["completed"] == lv["requests"]
          and lv["atm500x500"]["p99_ms"] <= SERVE_P99_TARGET_MS]
    best = max(ok, key=lambda lv: lv["offered_req_per_s"]) if ok else None
    target = None if best is None else {
        "p99_target_ms": SERVE_P99_TARGET_MS,
        "offered_req_per_s": best["offered_req_per_s"], "achieved_req_per_s": best["achieved_req_per_s"],
        "probabilities_per_s": best["probabilities_per_s"], "atm500x500": best["atm500x500"],
        "fraction_of_highest_throughput": round(best["achieved_req_per_s"] / top["achieved_req_per_s"], 3)}
    if knee is None:
        return {"capacity_req_per_s": round(cap, 1), "sustained": None, "highest_throughput": sat,
                "highest_load_meeting_p99_target_500x500": target}
    out = {"capacity_req_per_s": round(cap, 1), "highest_throughput": sat,
           "highest_load_meeting_p99_target_500x500": target,
           "offered_req_per_s": knee["offered_req_per_s"],
           "achieved_req_per_s": knee["achieved_req_per_s"],
           "probabilities_per_s": knee["probabilities_per_s"],
           "p50_ms": knee["p50_ms"], "p99_ms": knee["p99_ms"],
           "atm500x500": knee.get("atm500x500"),
           "clocks": knee.get("clocks")}
    return out


def run_serve(args, rank, world):
    """Serving workload: open-loop Poisson arrivals from 64 chains over request sizes {atm
    200^2, 500^2, 2000^2; beam 1e4, 1e5}, swept over offered loads up to past the server's
    capacity; p50/p99 latency and probabilities/s per level."""
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    fractions = args.serve_loads or [0.2, 0.4, 0.6, 0.8, 1.0, 1.2, 1.4, 1.6, 1.8, 2.0]
    cap, levels, knee, kinds, bursts = serve_sweep(dev, fractions, args.serve_seconds, dev)
    top = knee or levels[0]
    line = {
        "metric": "serving: probabilities/s at the highest sustained offered load (open-loop "
                  "Poisson, 64 chains), p50/p99 latency vs offered load",
        "value": world * top["probabilities_per_s"], "unit": "probabilities/s", "n_gpus": world,
        "steps": len(levels), "warmup": 1, "ms_per_step": args.serve_seconds * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded parameter sets and arrivals; PREM 4-layer, h=22 km; beam "
                "rho=2.6, L=1300 km)",
        "config": {"workload": "serve", "chains": 64, "arrivals": "open-loop Poisson",
                   "request_sizes": [k[0] for k in kinds], "pool_bytes": 16 << 30,
                   "max_bins_per_launch": 8_000_000, "scheduling": "smallest-first, 4 ms aging",
                   "seconds_per_level": args.serve_seconds},
        "serve": dict(serve_summary(cap, knee, kinds, levels),
                      capacity_bursts_req_per_s=[round(x, 1) for x in bursts]),
        "latency_p99_atm500_at_knee_ms": (knee or {}).get("atm500x500", {}).get("p99_ms"),
        "levels": levels,
        "clocks": top["clocks"],
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(workload("serve"), seconds=args.cpu_seconds)
    return line


def make_pair(w, prec, m):
    """Neutrino and antineutrino handles of one workload and parameter set."""
    props = []
    for knu in (1, -1):
        p = make_propagator(w, prec)
        set_params(p, m, knu)
        props.append(p)
    return props


def time_device_steps(props, stream, flush, steps, warmup, gpu, world):
    """Device-resident steps: neutrino and antineutrino on two streams forked from and joined
    back into `stream`, as a caller with two handles would run them (one type's eigen-table
    kernel overlaps the other's per-bin kernel).  The host queues the steps back to back;
    each is timed with CUDA events on `stream`, with the L2 flushed (untimed) before it.
    Returns (per-step ms, clock record)."""
    import torch
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

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(gpu) as clk:
        for k in range(steps):
            flush.add_(1.0)
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    return [a.elapsed_time(b) for a, b in ev], clk.summary()


def serial_kernel_times(props, sptr, flush, n):
    """Per-launch kernel durations from the ABI's own CUDA events, the two types one after
    the other on one stream with the L2 flushed before each: (table ms, per-bin ms) means."""
    import torch
    eig, bins = [], []
    for p in props:
        p.set_profiling(True)
    for _ in range(n):
        for t, p in enumerate(props):
            flush.add_(1.0)
            p.calculate_async(t, sptr)
            a, b = p.kernel_times()
            eig.append(a)
            bins.append(b)
    for p in props:
        p.set_profiling(False)
    torch.cuda.synchronize()
    return float(np.mean(eig)), float(np.mean(bins))


def oracle_full(w, m):
    """The CPU oracle on the whole grid, neutrino and antineutrino (reference CPU layout)."""
    from oracle.oracle import Mixing as OMix, Oracle
    orc = Oracle()
    nt = os.cpu_count() or 1
    refs = []
    for anti, knu in ((False, 1), (True, -1)):
        mix = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu)
        if w["kind"] == "atmos":
            refs.append(orc.atmos(mix, anti, w["cz"], w["en"], *w["model"], w["h"], nthreads=nt))
        else:
            refs.append(orc.beam(mix, anti, w["en"], w["rho"], w["L"], nthreads=nt))
    return refs


def channel_errors(props, refs):
    """Max |GPU - oracle| of each of the nine channels (index a*3+b = P(a->b)), per neutrino
    type, over every bin of the grid."""
    out = {}
    for name, p, ref in zip(("nu", "nubar"), props, refs):
        res = p.result()  # [9][nc][ne] (atmospheric) or [9][ne] (beam), device precision
        errs = []
        for c in range(9):
            errs.append(float(np.abs(res[c].astype(np.float64) - ref[..., c]).max()))
        out[name] = errs
    return out


def fp64_arm(w, m, stream, flush, steps, warmup, gpu, world, refs, peaks, flops_launch):
    """The plain FP64 kernels on the same grid, parameters and step structure as the mixed
    arm: device probabilities/s, kernel times, FP64 roofline and per-channel errors."""
    props = make_pair(w, "fp64", m)
    step_ms, clocks = time_device_steps(props, stream, flush, steps, warmup, gpu, world)
    t_ms = max_over_ranks(float(np.mean(step_ms)), world, "cuda")
    nbins = len(w["en"]) * (len(w["cz"]) if w["kind"] == "atmos" else 1)
    probs_step = 9 * nbins * N_TYPES
    eig_ms, kern_ms = serial_kernel_times(props, stream.cuda_stream, flush, 3)
    out = {"value": world * probs_step / (t_ms * 1e-3), "unit": "probabilities/s",
           "ms_per_step": t_ms, "steps": steps,
           "kernel": "atmos_f64_kernel" if w["kind"] == "atmos" else "beam_f64_kernel",
           "kernel_ms": round(kern_ms, 4), "eigen_table_ms": round(eig_ms, 4)}
    if peaks.get("fp64"):
        achieved = flops_launch / (kern_ms * 1e-3) / 1e12
        out["roofline"] = {"bound": "fp64", "achieved": round(achieved, 3),
                           "peak": round(peaks["fp64"], 3), "unit": "TFLOP/s",
                           "frac": round(achieved / peaks["fp64"], 4),
                           "frac_incl_table": round(flops_launch / ((kern_ms + eig_ms) * 1e-3)
                                                    / 1e12 / peaks["fp64"], 4),
                           **ncu_pipe(w.get("name", ""), "fp64")}
    if refs is not None:
        errs = channel_errors(props, refs)
        out["max_abs_err_per_channel"] = errs
        out["max_abs_err_vs_oracle"] = max(max(v) for v in errs.values())
    out["clocks"] = clocks
    for p in props:
        p.close()
    return out


def reference_gpu(w, m, steps, refs, sample_every=40, timeout=600):
    """The reference's own FP64 CUDA propagator (AtmosCudaPropagatorSingle, compiled from the
    reference tree by `make -C oracle refgpu`) on the same grid and parameters, timed through
    its public, synchronous calculateProbabilities in a child process; every
    sample_every-th cosine row read back through getProbability and checked against the
    oracle."""
    from oracle.oracle import Reference
    exe = Reference.GPU_BENCH
    if not os.path.exists(exe):
        return {"unavailable": "no reference source tree here (CP3_REFERENCE_DIR or "
                               "baseline/_ref), so the reference's CUDA propagator was not built"}
    with tempfile.TemporaryDirectory() as d:
        inp, outb = os.path.join(d, "in.txt"), os.path.join(d, "sample.bin")
        with open(inp, "w") as f:
            f.write(f"kind {w['kind']}\nsteps {steps}\nwarmup 1\n")
            f.write("params %r %r %r %r %r %r\n" % (m.theta12, m.theta13, m.theta23, m.dcp,
                                                    m.dm12sq, m.dm23sq))
            if w["kind"] == "atmos":
                r, rho, ye = w["model"]
                f.write(f"height_km {w['h']!r}\nsample_every {sample_every}\n")
                f.write(f"cosines {len(w['cz'])} " + " ".join(repr(float(x)) for x in w["cz"]) + "\n")
                f.write(f"model {len(r)}\n" + "".join(f"{a!r} {b!r} {c!r}\n" for a, b, c in
                                                      zip(map(float, r), map(float, rho), map(float, ye))))
            else:
                f.write(f"rho {w['rho']!r}\nlength_km {w['L']!r}\n")
            f.write(f"energies {len(w['en'])} " + " ".join(repr(float(x)) for x in w["en"]) + "\n")
        try:
            r = subprocess.run([exe, inp, outb], capture_output=True, text=True, timeout=timeout)
        except subprocess.TimeoutExpired:
            return {"unavailable": f"the reference's CUDA propagator did not finish in {timeout} s"}
        try:
            res = json.loads(r.stdout.strip().splitlines()[-1])
        except (ValueError, IndexError):
            res = {}
        if r.returncode != 0 or "ms_per_call" not in res:
            return {"unavailable": f"the reference's CUDA propagator exited {r.returncode}: "
                                   + (res.get("error") or (r.stdout + r.stderr).strip()[-300:])}
        ms = np.asarray(res["ms_per_call"], dtype=np.float64)  # [step][nu, nubar]
        ne = len(w["en"])
        rows = len(w["cz"][::sample_every]) if w["kind"] == "atmos" else 1
        sample = np.fromfile(outb, dtype=np.float64)
    step_ms = float(np.mean(ms.sum(axis=1)))
    nbins = ne * (len(w["cz"]) if w["kind"] == "atmos" else 1)
    out = {"value": 9 * nbins * N_TYPES / (step_ms * 1e-3), "unit": "probabilities/s",
           "ms_per_step": step_ms, "ms_per_call": [round(float(x), 3) for x in ms.mean(axis=0)],
           "steps": int(len(ms)), "device": res.get("device"),
           "source": "the reference's AtmosCudaPropagatorSingle/BeamCudaPropagatorSingle "
                     "(calculateAtmosKernel / calculateBeamKernel, FP64), compiled from its own "
                     "sources for sm_103a with MaxNLayers raised to 64 through the constants "
                     "header's include guard; wall time of its synchronous calculateProbabilities",
           "timing": "one propagator per neutrino type, called one after the other"}
    if refs is not None and sample.size == 2 * rows * ne * 9:
        sample = sample.reshape(2, rows, ne, 9)
        errs = []
        for t in range(2):
            ref = refs[t][::sample_every] if w["kind"] == "atmos" else refs[t][None]
            errs.append(float(np.abs(sample[t] - ref).max()))
        out["max_abs_err_vs_oracle"] = max(errs)
        out["checked"] = (f"every {sample_every}th cosine row" if w["kind"] == "atmos"
                          else "every energy")
    return out


def reference_gpu_batch(w, n_sets=16, steps=3, sample_every=40, timeout=900):
    """The reference's own FP64 CUDA propagators on the first n_sets parameter sets of a batched
    workload, as a caller without batching runs them: one propagator per problem (created
    before the timed region), calculateProbabilities on each in turn, in a child process.
    Every sample_every-th cosine row (atmospheric) or energy (beam) of every problem is read
    back through getProbability and checked against the oracle."""
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix, Oracle, Reference
    exe = Reference.GPU_BENCH
    if not os.path.exists(exe):
        return {"unavailable": "no reference source tree here (CP3_REFERENCE_DIR or "
                               "baseline/_ref), so the reference's CUDA propagator was not built"}
    fl = lambda xs: " ".join(repr(float(x)) for x in xs)  # noqa: E731
    probs = []  # (kind, set, anti, grid or (en, L))
    with tempfile.TemporaryDirectory() as d:
        inp, outb = os.path.join(d, "in.txt"), os.path.join(d, "sample.bin")
        with open(inp, "w") as f:
            f.write(f"kind batch\nsteps {steps}\nwarmup 1\nsample_every {sample_every}\n")
            if w["model"] is not None:
                r, rho, ye = w["model"]
                f.write(f"height_km {w['h']!r}\nmodel {len(r)}\n" + "".join(
                    f"{a!r} {b!r} {c!r}\n" for a, b, c in zip(map(float, r), map(float, rho), map(float, ye))))
            for k in range(min(n_sets, len(w["sets"]))):
                m = w["sets"][k]
                par = "%r %r %r %r %r %r" % (m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq)
                for anti in (0, 1):
                    if w["model"] is not None:
                        nc, ne = w["grids"][k]
                        cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
                        f.write(f"problem atmos {par} {anti} cosines {nc} {fl(cz)} energies {ne} {fl(en)}\n")
                        probs.append(("atmos", m, anti, (cz, en)))
                    else:
                        bw = w["beam"]
                        for L in bw["L"]:
                            f.write(f"problem beam {par} {anti} rho {bw['rho']!r} length_km {float(L)!r} "
                                    f"energies {len(bw['en'])} {fl(bw['en'])}\n")
                            probs.append(("beam", m, anti, (bw["en"], float(L))))
        try:
            r = subprocess.run([exe, inp, outb], capture_output=True, text=True, timeout=timeout)
        except subprocess.TimeoutExpired:
            return {"unavailable": f"the reference's CUDA propagator did not finish in {timeout} s"}
        try:
            res = json.loads(r.stdout.strip().splitlines()[-1])
        except (ValueError, IndexError):
            res = {}
        if r.returncode != 0 or "ms_per_step" not in res:
            return {"unavailable": f"the reference's CUDA propagator exited {r.returncode}: "
                                   + (res.get("error") or (r.stdout + r.stderr).strip()[-300:])}
        sample = np.fromfile(outb, dtype=np.float64)
    step_ms = float(np.mean(res["ms_per_step"]))
    out = {"value": 9 * res["bins"] / (step_ms * 1e-3), "unit": "probabilities/s",
           "ms_per_step": step_ms, "steps": len(res["ms_per_step"]), "problems": res["problems"],
           "device": res.get("device"),
           "source": "the reference's AtmosCudaPropagatorSingle/BeamCudaPropagatorSingle (FP64), "
                     "compiled from its own sources for sm_103a with MaxNLayers raised to 64; "
                     "wall time of its synchronous calculateProbabilities",
           "timing": f"the first {min(n_sets, len(w['sets']))} parameter sets, nu and nubar"
                     + ("" if w["model"] is not None else ", both baselines")
                     + ": one propagator per problem, called one after the other (the reference "
                       "has no batching)"}
    orc, err, pos = Oracle(), 0.0, 0
    nt = os.cpu_count() or 1
    for kind, m, anti, g in probs:
        om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, -1 if anti else 1)
        if kind == "atmos":
            cz, en = g
            rows = cz[::sample_every]
            n = len(rows) * len(en) * 9
            ref = orc.atmos(om, bool(anti), rows, en, *w["model"], w["h"], nthreads=nt)
            got = sample[pos:pos + n].reshape(len(rows), len(en), 9)
        else:
            en, L = g
            es = en[::sample_every]
            n = len(es) * 9
            ref = orc.beam(om, bool(anti), es, w["beam"]["rho"], L, nthreads=nt)
            got = sample[pos:pos + n].reshape(len(es), 9)
        pos += n
        if got.size == ref.size:
            err = max(err, float(np.abs(got - ref).max()))
    if pos == sample.size:
        out["max_abs_err_vs_oracle"] = err
        out["checked"] = (f"every {sample_every}th " + ("cosine row" if w["model"] is not None else "energy")
                          + " of every problem run")
    return out


def run_ours(args, rank, world):
    import torch

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if args.workload == "serve":
        return run_serve(args, rank, world)
    w = workload(args.workload, rank)
    if w["kind"] == "batch":
        if args.precision == "fp64":
            return run_batch_fp64(args, w, rank, world)
        return run_batch(args, w, rank, world)
    w["name"] = args.workload
    prec = args.precision
    # weak scaling: each rank propagates its own parameter set over the full grid
    m = rank_parameter_set(rank, world)
    props = make_pair(w, prec, m)
    # A dedicated stream: kernels, events and the L2 flush are all ordered on it (the legacy
    # default stream's handle is 0, which the C ABI reads as "the handle's own stream").
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    assert sptr != 0
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

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
    step_ms, clocks = time_device_steps(props, stream, flush, args.steps, args.warmup, dev, world)
    t_ms = max_over_ranks(float(np.mean(step_ms)), world, "cuda")
    value = world * probs_step / (t_ms * 1e-3)

    # The roofline's kernel durations come from a second, serial pass (the two types one
    # after the other on one stream, L2 flushed before each): in the timed steps the types
    # overlap, so each kernel's wall time there includes the other's.
    eig_ms, kernel_ms = serial_kernel_times(props, sptr, flush, max(3, args.steps))

    # end to end through the public API: grid H2D from pinned memory, compute, full D2H
    is_float = prec == "mixed"
    # two page-locked result buffers per type, used in turn: a step's download may still be
    # in flight while the host queues the next step
    host_out = [[torch.empty(bytes_out_launch // (4 if is_float else 8),
                             dtype=torch.float32 if is_float else torch.float64, pin_memory=True)
                 for _ in range(2)] for _ in props]
    en_pinned = torch.from_numpy(np.asarray(w["en"], dtype=np.float64)).pin_memory()
    cz_pinned = (torch.from_numpy(np.asarray(w["cz"], dtype=np.float64)).pin_memory()
                 if w["kind"] == "atmos" else None)

    # neutrino and antineutrino each on their own pair of streams, used in turn, each step
    # computed in row pieces whose downloads (on the handle's copy stream) overlap the next
    # piece's compute (cp3_calculate_to_host_async).  Steps are queued back to back, as a
    # fitter pipelines consecutive evaluations: a step's setters and compute are queued while
    # the previous step's download is still on the link.  The handle orders its uploads,
    # computes and copies on the device (a row piece is recomputed once its previous copy
    # has left), and the step's stream waits for its download, so the two streams let a step
    # compute behind the previous step's download.  The timed region ends when the last
    # step's results are in host memory.
    e2e_streams = [[torch.cuda.Stream(), torch.cuda.Stream()] for _ in props]

    def e2e_step(k, wait):
        for t, p in enumerate(props):
            p.setEnergyList(en_pinned.numpy())
            if cz_pinned is not None:
                p.setCosineList(cz_pinned.numpy())
            sp = e2e_streams[t][k % 2].cuda_stream
            p.calculate_to_host_async(t, host_out[t][k % 2].data_ptr(), 0, sp)
        if wait:
            for st in e2e_streams:
                st[k % 2].synchronize()

    for k in range(max(1, args.warmup)):
        e2e_step(k, True)
    torch.cuda.synchronize()
    # Five trials of the K steps, the median trial reported (an occasional slowdown of the
    # shared machine's device-to-host link would otherwise decide a loop this short), and
    # the same steps with the host waiting for each step's results before the next.
    trials, trials_sync = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        for k in range(args.steps):
            e2e_step(k, False)
        for pair in e2e_streams:
            for st in pair:
                st.synchronize()
        trials.append((time.perf_counter() - t0) * 1e3 / args.steps)
        t0 = time.perf_counter()
        for k in range(args.steps):
            e2e_step(k, True)
        trials_sync.append((time.perf_counter() - t0) * 1e3 / args.steps)
    e2e_ms = max_over_ranks(statistics.median(trials), world, "cuda")
    e2e_ms_sync = max_over_ranks(statistics.median(trials_sync), world, "cuda")
    # bytes that cross the link: the energy lists; an unchanged cosine list is recognised
    # on the host (one memcmp) and not uploaded again
    h2d = len(w["en"]) * 8 * len(props)
    d2h = bytes_out_launch * len(props)

    peaks = fma_peaks(dev)
    peak = peaks.get("fp32") if prec == "mixed" else peaks.get("fp64")
    achieved = flops_launch / (kernel_ms * 1e-3) / 1e12
    roofline = {
        "bound": "fp32" if prec == "mixed" else "fp64",
        "achieved": round(achieved, 3),
        "peak": round(peak, 3),
        "unit": "TFLOP/s",
        "frac": round(achieved / peak, 4),
        # the canonical count includes the per-segment eigen-solve, which these kernels do
        # once per (density class, energy) in the table kernel: charging its time as well
        "frac_incl_table": round(flops_launch / ((kernel_ms + eig_ms) * 1e-3) / 1e12 / peak, 4),
        "traffic": ncu_traffic(args.workload, prec, bytes_out_launch)[0],
        "traffic_note": ncu_traffic(args.workload, prec, bytes_out_launch)[1],
        **ncu_pipe(args.workload, prec),
        "peak_source": "live FMA-chain microbenchmark in this run (cp3_peaks.cu); the pool's "
                       "measured HBM/bf16 peaks do not apply to scalar FP pipes",
        "kernel": "atmos_mixed_kernel" if (w["kind"] == "atmos" and prec == "mixed") else
                  ("atmos_f64_kernel" if w["kind"] == "atmos" else
                   ("beam_mixed_kernel" if prec == "mixed" else "beam_f64_kernel")),
        "kernel_ms": round(kernel_ms, 4),
        "eigen_table_ms": round(eig_ms, 4),
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
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "steps_queued": "back to back, results in two page-locked buffers per type in "
                                "turn, two streams per type in turn",
                "trials_ms_per_step": [round(t, 4) for t in trials],
                "trials_ms_per_step_waiting_each_step": [round(t, 4) for t in trials_sync],
                "timing": "median of 5 trials of the K steps",
                "ms_per_step_waiting_each_step": e2e_ms_sync,
                "link": link_summary(d2h, e2e_ms, d2h_link())},
        "gpu_launches": args.steps * len(props) * (2 if w["kind"] == "atmos" else 1),
        "roofline": roofline,
        "peaks_tflops": peaks,
    }

    # parity of this run: every bin of both types against the CPU oracle, per channel
    refs = oracle_full(w, m) if rank == 0 else None
    if refs is not None:
        errs = channel_errors(props, refs)
        line["max_abs_err_vs_oracle"] = max(max(v) for v in errs.values())
        line["max_abs_err_per_channel"] = dict(errs, channels="a*3+b = P(a->b): e_e, e_m, e_t, "
                                               "m_e, m_m, m_t, t_e, t_m, t_t",
                                               bins="every bin of the grid")
    line["clocks"] = clocks
    for p in props:
        p.close()
    del host_out

    if prec == "mixed" and not args.no_fp64:
        fp = fp64_arm(w, m, stream, flush, args.steps, args.warmup, dev, world, refs, peaks,
                      flops_launch)
        line["fp64"] = fp
        line["mixed_over_fp64"] = round(value / fp["value"], 2)
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        line["reference_fp64_gpu"] = reference_gpu(w, m, 3, refs)
        if "value" in line["reference_fp64_gpu"]:
            line["mixed_over_reference_fp64_gpu"] = round(value / line["reference_fp64_gpu"]["value"], 1)
    if args.workload == "atmos59" and not args.no_serve:
        cap, levels, knee, kinds, bursts = serve_sweep(dev, [0.5, 0.8, 1.0, 1.2, 1.4, 1.6, 1.8], 1.0, dev)
        line["serve"] = dict(serve_summary(cap, knee, kinds, levels),
                             capacity_bursts_req_per_s=[round(x, 1) for x in bursts],
                             workload="open-loop Poisson arrivals from 64 chains, sizes "
                                      + ", ".join(k[0] for k in kinds) + "; PREM 4-layer",
                             levels=[{k: lv[k] for k in ("fraction_of_capacity", "offered_req_per_s",
                                                         "achieved_req_per_s", "p50_ms", "p99_ms")}
                                     for lv in levels])
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, seconds=args.cpu_seconds)
    return line


class CpuPath:
    """The CPU implementation timed beside the GPU: the reference's own CpuPropagator<double>
    (AtmosCpuPropagator / BeamCpuPropagator built from its headers into
    oracle/_ref/libcp3ref_fast.so, MaxNLayers raised to 64) where it was compiled, else the C
    restatement (oracle/_build/libcp3oracle_fast.so).  Both use OpenMP over cosines."""

    def __init__(self):
        from oracle.oracle import Oracle, Reference
        if Reference.available(fast=True):
            self.impl, self.kind = Reference(fast=True), "reference"
            self.what = ("the reference's own AtmosCpuPropagator<double>/BeamCpuPropagator<double> "
                         "compiled from its headers (-O3 -fopenmp, MaxNLayers raised to 64 "
                         "through the constants header's include guard); time of "
                         "calculateProbabilities, all host threads")
        else:
            self.impl, self.kind = Oracle(fast=True), "port"
            self.what = ("C restatement of the reference CpuPropagator<double> (oracle/"
                         "cp3_oracle.c, OpenMP over cosines, -O3), all host threads; the "
                         "reference's own build needs its source tree, absent on this host")

    def seconds(self, w, m, nthreads):
        """Compute seconds of one single-grid job, neutrino and antineutrino."""
        from oracle.oracle import Mixing as OMix
        total = 0.0
        for anti, knu in ((False, 1), (True, -1)):
            mix = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu)
            if self.kind == "reference":
                if w["kind"] == "atmos":
                    total += self.impl.atmos(mix, anti, w["cz"], w["en"], *w["model"], w["h"],
                                             nthreads=nthreads, reps=1)[1]
                else:
                    for L in np.atleast_1d(w["L"]):
                        total += self.impl.beam(mix, anti, w["en"], w["rho"], float(L),
                                                nthreads=nthreads, reps=1)[1]
                continue
            t0 = time.perf_counter()
            if w["kind"] == "atmos":
                self.impl.atmos(mix, anti, w["cz"], w["en"], *w["model"], w["h"], nthreads=nthreads)
            else:
                for L in np.atleast_1d(w["L"]):
                    self.impl.beam(mix, anti, w["en"], w["rho"], float(L), nthreads=nthreads)
            total += time.perf_counter() - t0
        return total


def cpu_run(w, cpu, nthreads, m=None):
    """Probabilities/s of the CPU implementation on one single-grid job, nu and nubar."""
    from cudaprob3_gb300 import earth
    return job_probs(w) / max(cpu.seconds(w, m or earth.NOMINAL, nthreads), 1e-12)


def cpu_sample(w, seconds, cpu=None, nthreads=1):
    """A bounded slice of the workload for the CPU, sized from a short probe run to take
    about ``seconds`` of compute: every k-th cosine row (keeps the distribution of shells
    crossed) or a contiguous block of beam energies."""
    if w["kind"] == "atmos":
        stride = max(1, len(w["cz"]) // 8)
        if cpu is not None:
            # a warm-up (library, thread pool), then a probe of four rows per thread
            stride = max(1, len(w["cz"]) // (4 * nthreads))
            probe = dict(w, cz=w["cz"][::stride])
            cpu_run(dict(probe, cz=probe["cz"][:nthreads]), cpu, nthreads)
            rows_per_s = cpu_run(probe, cpu, nthreads) / (job_probs(probe) / len(probe["cz"]))
            # enough rows that the dynamic schedule keeps every thread busy
            rows = max(8 * nthreads, min(len(w["cz"]), int(seconds * rows_per_s)))
            stride = max(1, len(w["cz"]) // rows)
        sub = w["cz"][::stride]
        if stride == 1:
            return dict(w, cz=sub), f"the whole grid ({len(sub)} x {len(w['en'])} bins), nu+nubar"
        return dict(w, cz=sub), f"every {stride}th cosine row ({len(sub)} x {len(w['en'])} bins), nu+nubar"
    n = len(w["en"])
    if cpu is not None:
        probe = dict(w, en=w["en"][:20000])
        cpu_run(probe, cpu, nthreads)  # warm-up
        per_energy = 1.0 / (cpu_run(probe, cpu, nthreads) / (job_probs(probe) / 20000))
        n = max(20000, min(n, int(seconds / max(per_energy, 1e-12))))
    return dict(w, en=w["en"][:n]), f"{n} energies, nu+nubar"


def cpu_jobs(w, seconds, cpu, nthreads):
    """The CPU's share of a workload: (list of (single-grid workload, parameter set), text).
    Single grids are sliced by cpu_sample; batched workloads take their first parameter sets
    on their own grids, as many as fit about ``seconds``; serving takes 500 x 500 PREM-4
    requests (the size its latency target is quoted for)."""
    from cudaprob3_gb300 import earth
    if w["kind"] in ("atmos", "beam"):
        sw, desc = cpu_sample(w, seconds, cpu, nthreads)
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
        cpu_run(job[0], cpu, nthreads, job[1])
        jobs.append(job)
        if time.perf_counter() - t0 >= seconds:
            break
    return jobs, f"the first {len(jobs)} {what}, nu+nubar"


def job_probs(w):
    """Probabilities of one single-grid job, nu and nubar."""
    if w["kind"] == "atmos":
        return 9 * N_TYPES * len(w["cz"]) * len(w["en"])
    return 9 * N_TYPES * len(w["en"]) * len(np.atleast_1d(w["L"]))


def run_jobs(jobs, cpu, nthreads):
    """Probabilities/s over a list of jobs (one pass; compute time only)."""
    from cudaprob3_gb300 import earth
    secs = sum(cpu.seconds(w, m or earth.NOMINAL, nthreads) for w, m in jobs)
    return sum(job_probs(w) for w, _ in jobs) / max(secs, 1e-12)


def cpu_baseline(w, seconds=2.0):
    cpu = CpuPath()
    cores = os.cpu_count() or 1
    jobs, desc = cpu_jobs(w, seconds, cpu, cores)  # the sizing run also warms up
    rate = run_jobs(jobs, cpu, cores)
    return {"value": rate, "unit": "probabilities/s", "cores": cores, "kind": cpu.kind,
            "sample": desc + "; " + cpu.what}


def run_reference(args):
    """The reference arm: the reference's own CPU propagators (where its sources were found
    and compiled; else the C restatement) on the host cores, on a bounded sample."""
    from oracle import oracle
    oracle.build()
    oracle.build_reference(gpu=False)
    w = workload(args.workload)
    cpu = CpuPath()
    cores = os.cpu_count() or 1
    jobs, desc = cpu_jobs(w, args.cpu_seconds, cpu, cores)
    for _ in range(max(0, args.warmup - 1)):  # the sizing pass was the first warm-up
        run_jobs(jobs, cpu, cores)
    rates = [run_jobs(jobs, cpu, cores) for _ in range(args.steps)]
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
                         "kind": cpu.kind, "sample": desc + "; " + cpu.what},
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
    ap.add_argument("--serve-seconds", type=float, default=1.5,
                    help="seconds of arrivals per offered-load level")
    ap.add_argument("--serve-loads", type=float, nargs="*", default=None,
                    help="offered loads as fractions of the measured capacity, one level each")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=2.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="leave out the plain FP64 arm of the single-grid workloads")
    ap.add_argument("--no-serve", action="store_true",
                    help="leave out the serving sweep of the default workload")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="leave out the reference's own FP64 CUDA propagator")
    ap.add_argument("--batch-sets", type=int, default=0,
                    help="parameter sets of the batched workloads (default: the configuration's)")
    ap.add_argument("--shape", type=int, nargs=3, default=None,
                    metavar=("ROWS_PER_TILE", "BLOCKS_PER_SM", "BEAM_CHUNK"),
                    help="batched workloads: this tile shape instead of the autotuner's "
                         "(so that a profiler captures the launch it is asked for)")
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
