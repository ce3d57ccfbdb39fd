"""Benchmark of the GB300 recrystallization growth step (one JSON line on stdout).

Workload (one bench "step" = one complete growth run): a 512^3 domain of 20,000
periodic-Voronoi deformed grains (uniform orientations, lognormal rho, mean
1e15 m^-2, sigma 0.3) with 50,000 site-saturated nuclei at distinct uniform
sites, Sebald-Gottstein mobility, T = 1000 K, FP64 fill, run from nucleation
until X > 0.99.  Inputs are synthetic and seeded (rank r uses seed r).

  value   front-cell updates/s = sum of Sv over all steps of all runs / time,
          inputs resident in HBM (score_restart + place_nuclei + run_until),
          timed with CUDA events on the library's stream, max over ranks.
  e2e     same metric through the C ABI from pinned host buffers: every run
          copies the domain in (score_load_domain) and the labels out.
  roofline  grow kernel (the dominant kernel): algorithmic bytes (29 B per FP64
          front-cell update) / its event-timed duration, against the measured
          HBM copy bandwidth.
  cpu_baseline  the C oracle (single thread) on a bounded 256^3 sample of the
          same workload (same grain and nucleus densities), run to X > 0.99.

`--impl reference` times the reference's CPU path instead: the oracle port (the
SCORE reference cannot be compiled on this host) as independent same-density
192^3 domains, one per host core, like the reference's MPI ensemble of solitary
units; rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from concurrent.futures import ProcessPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_EDGE = 512
N_GRAINS = 20000
N_NUCLEI = 50000
X_TARGET = 0.99
# algorithmic bytes of one front-cell update in k_grow_fill: FP64 reads the infector byte,
# the cached increment and the fill and writes the fill (1 + 8 + 8 + 8); FP32+Kahan
# reads byte, velocity factor, fill and compensation and writes fill and compensation
BYTES_PER_UPDATE = {0: 25.0, 1: 17.0}
METRIC = "front-cell updates/s (RX growth step to X=0.99)"
WORKLOAD = "512^3 Voronoi domain, 20000 deformed grains, 50000 site-saturated nuclei, FP64, T=1000K, until X>0.99"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    backend = "nccl"
    try:
        import torch
        if not torch.cuda.is_available():
            backend = "gloo"
    except Exception:
        backend = "gloo"
    dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def spec_for(n: int, precision: int = 0):
    import score_gb300 as sg
    return sg.UdsSpec(nx=n, ny=n, nz=n, precision=precision)


def read_params(n: int, precision: int = 0):
    import score_gb300 as sg
    with tempfile.TemporaryDirectory() as td:
        return sg.read_uds(spec_for(n, precision).write(Path(td) / "bench.uds"))


def measured_peak_gbs():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in self.path.read_text().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def pinned_copy(a: np.ndarray) -> np.ndarray:
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t.numpy()


def oracle_sample(args):
    """One same-density sample run on the CPU oracle (process-pool worker)."""
    n, seed = args
    sys.path.insert(0, str(ROOT))
    import score_gb300 as sg
    import oracle
    f = (n / N_EDGE) ** 3
    d = sg.generate_domain(n, n, n, max(1, round(N_GRAINS * f)), max(1, round(N_NUCLEI * f)), seed=seed)
    p = read_params(n)
    t0 = time.perf_counter()
    r = oracle.run(p, d, x_target=X_TARGET)
    el = time.perf_counter() - t0
    return int(r["trace"]["Sv"].sum()), r["seconds"], el


def cpu_baseline(n: int = 256) -> dict:
    sv, loop_s, _ = oracle_sample((n, 1000))
    return {"value": sv / loop_s, "unit": "updates/s", "cores": 1, "kind": "port",
            "sample": f"C oracle, 1 thread, {n}^3 domain at the workload's grain/nucleus densities, to X>0.99 "
                      f"({sv} updates in {loop_s:.2f} s)"}


def run_reference_arm(args) -> None:
    """The reference's CPU algorithm on the host cores; under torchrun only rank 0
    works and prints, the other ranks exit at once (no process group needed)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build_oracle()
    cores = os.cpu_count() or 1
    n = 192
    def one_round(k):
        with ProcessPoolExecutor(max_workers=cores, mp_context=__import__("multiprocessing").get_context("spawn")) as ex:
            t0 = time.perf_counter()
            res = list(ex.map(oracle_sample, [(n, 5000 + 131 * k + i) for i in range(cores)]))
            return sum(r[0] for r in res), time.perf_counter() - t0
    for w in range(args.warmup):
        one_round(w)
    tot_sv, tot_s = 0, 0.0
    for k in range(args.steps):
        sv, s = one_round(100 + k)
        tot_sv += sv
        tot_s += s
    v = tot_sv / tot_s
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "updates/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": f"{cores} independent {n}^3 domains per step at the same densities"},
            "cpu_baseline": {"value": v, "unit": "updates/s", "cores": cores, "kind": "port",
                             "sample": f"C oracle (the reference's algorithm restated; the reference itself does not build on this host), "
                                       f"{cores} processes x one {n}^3 domain each, to X>0.99"},
            "e2e": {"value": v, "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--edge", type=int, default=N_EDGE)
    ap.add_argument("--precision", type=int, default=0, help="0 FP64 (bit-exact), 1 FP32+Kahan")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end runs (profiling captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    rank, world, local = dist_env()
    dist = init_dist(world)
    import score_gb300 as sg
    sg.build()
    n = args.edge
    f = (n / N_EDGE) ** 3
    ngr, nnuc = max(1, round(N_GRAINS * f)), max(1, round(N_NUCLEI * f))
    d = sg.generate_domain(n, n, n, ngr, nnuc, seed=rank)
    p = read_params(n, args.precision)
    gm = sg.GrowthMachine(p, device=local)
    gm.load_domain(d)

    def one_run():
        gm.restart()
        gm.place_nuclei()
        tr = gm.run_until(X_TARGET)
        tm = gm.timing()
        one_run.misses = sum(s.p_misses for s in tr)
        return sum(s.Sv for s in tr), len(tr), tm

    for _ in range(args.warmup):
        one_run()
    barrier(dist)
    launches0 = gm.timing().kernel_launches
    tot_sv, tot_steps, run_ms, grow_bytes, grow_launches = 0, 0, 0.0, 0.0, 0
    phase = {"grow_ms": 0.0, "fill_ms": 0.0, "claim_ms": 0.0, "commit_ms": 0.0, "host_ms": 0.0, "wait_ms": 0.0,
             "weights_ms": 0.0}
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            sv, ns, tm = one_run()
            tot_sv += sv
            tot_steps += ns
            run_ms += tm.run_ms
            grow_bytes += tm.grow_bytes
            grow_launches += tm.grow_launches
            for k in phase:
                phase[k] += getattr(tm, k)
    fill_ms = phase["fill_ms"]
    launches = gm.timing().kernel_launches - launches0
    barrier(dist)
    t_max = reduce_max(dist, run_ms / 1e3)
    sv_all = reduce_sum(dist, float(tot_sv))
    value = sv_all / t_max

    # end to end through the C ABI: pinned host inputs in, labels out, every run
    e_value, h2d, d2h = None, 0, 0
    if not args.no_e2e:
        pin = [pinned_copy(x) for x in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub)]
        pd = sg.Domain(n, n, n, *pin)
        lab = pinned_copy(np.empty((n, n, n), dtype=np.uint32))
        h2d = sum(x.nbytes for x in pin)
        d2h = lab.nbytes
        e2e_runs = max(1, min(args.steps, 3))
        gm.load_domain(pd)
        gm.place_nuclei()
        gm.run_until(X_TARGET)
        gm.labels(lab)
        barrier(dist)
        e_sv, t0 = 0, time.perf_counter()
        for _ in range(e2e_runs):
            gm.load_domain(pd)
            gm.place_nuclei()
            tr = gm.run_until(X_TARGET)
            gm.labels(lab)
            e_sv += sum(s.Sv for s in tr)
        e_s = time.perf_counter() - t0
        barrier(dist)
        e_s = reduce_max(dist, e_s)
        e_value = reduce_sum(dist, float(e_sv)) / e_s
    gm.close()

    if rank == 0:
        peak, peak_kind = measured_peak_gbs()
        bpu = BYTES_PER_UPDATE[args.precision]
        achieved = grow_bytes / (fill_ms / 1e3) / 1e9 if fill_ms > 0 else 0.0
        traffic = None
        tf = ROOT / "profiles" / "grow_traffic.json"
        if tf.exists():
            try:
                tj = json.loads(tf.read_text())
                traffic = tj["dram_bytes_per_update"] * (tot_sv / max(1, grow_launches))
            except Exception:
                traffic = None
        line = {
            "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": run_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == 0 else "f32+kahan", "data": "synthetic",
            "config": {"workload": WORKLOAD if n == N_EDGE else f"{n}^3 at the 512^3 workload's densities",
                       "cells": n ** 3, "grains": ngr, "nuclei": nnuc, "growth_steps_per_run": tot_steps // args.steps,
                       "updates_per_run": tot_sv // args.steps, "time_to_X099_ms": run_ms / args.steps,
                       "l2": "inputs larger than L2 (grid alone 512 MiB)", "parallelism": f"{world} independent domains",
                       "phase_ms_per_run": {k: v / args.steps for k, v in phase.items()},
                       "host_weight_misses_per_run": getattr(one_run, "misses", None)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if peak else None, "traffic": traffic,
                         "kernel": "k_grow_fill", "bytes_per_update": bpu, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
            "e2e": {"value": e_value, "unit": "updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
