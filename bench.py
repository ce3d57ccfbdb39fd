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
  roofline  k_grow_fill (the dominant kernel): algorithmic bytes (25 B per FP64
          front-cell update: infector byte, cached increment, fill read and write;
          21 B FP32+Kahan: byte, velocity factor, fill and compensation read and write) / its event-timed duration, against the measured HBM
          copy bandwidth.
  cpu_baseline  the C oracle (single thread) on a bounded 256^3 sample of the
          same workload (same grain and nucleus densities), run to X > 0.99.

`--workload batch` times the batched ensemble instead (64 domains, edges uniform in
[64, 256] per axis), `--precision 1` the FP32+Kahan fill (with its error against the
FP64 path), `--autotune` picks the launch configuration first.

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
# (1 + 4 + 4 + 4 + 4 + 4)
BYTES_PER_UPDATE = {0: 25.0, 1: 21.0}
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


def spec_for(n: int, precision: int = 0, **kw):
    import score_gb300 as sg
    return sg.UdsSpec(nx=n, ny=n, nz=n, precision=precision, **kw)


def read_params(n: int, precision: int = 0, **kw):
    import score_gb300 as sg
    with tempfile.TemporaryDirectory() as td:
        return sg.read_uds(spec_for(n, precision, **kw).write(Path(td) / "bench.uds"))


# config of the recovery workload: rho(t) = rho0 / (1 + k t), k = 0.01 1/s, and Poisson
# incubation times at 1e3 nuclei/s
RECOVERY_K = "0.01"
NUCLEATION_RATE = 1000.0
# config of the pancake workload: 1024^3, 8,000 grains flattened 1:4:8, orientations around
# 3 texture components with 10 degree scatter, rho 1e14 / 5e15 (50/50), 200,000 nuclei
# preferentially on grain boundaries
PANCAKE = dict(edge=1024, grains=8000, nuclei=200000,
               gen=dict(aspect=(1.0, 4.0, 8.0), ori_mode=1, ncomp=3, scatter_deg=10.0, rho_mode=1, rho_lo=1e14,
                        rho_hi=5e15, site_mode=1, gb_fraction=0.8))


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


class PlainWorkload:
    """One cubic domain through GrowthMachine (the headline workload at --edge 512)."""

    def __init__(self, sg, args, rank, local):
        n = args.edge
        f = (n / N_EDGE) ** 3
        self.n, self.ngr, self.nnuc = n, max(1, round(N_GRAINS * f)), max(1, round(N_NUCLEI * f))
        self.recovery = args.workload == "recovery"
        self.pancake = args.workload == "pancake"
        if self.pancake:
            n = PANCAKE["edge"]
            self.n, self.ngr, self.nnuc = n, PANCAKE["grains"], PANCAKE["nuclei"]
            self.d = sg.generate_domain(n, n, n, self.ngr, self.nnuc, seed=rank, **PANCAKE["gen"])
            self.p = read_params(n, args.precision)
        elif self.recovery:
            self.d = sg.generate_domain(n, n, n, self.ngr, self.nnuc, seed=rank, nucleation_rate=NUCLEATION_RATE)
            self.p = read_params(n, args.precision, recovery=10, recovery_k=RECOVERY_K)
        else:
            self.d = sg.generate_domain(n, n, n, self.ngr, self.nnuc, seed=rank)
            self.p = read_params(n, args.precision)
        self.sg = sg
        self.gm = sg.GrowthMachine(self.p, device=local)
        self.gm.load_domain(self.d)
        self.tuned = self.gm.autotune(X_TARGET) if args.autotune else None
        self.misses = None

    def run(self):
        gm = self.gm
        gm.restart()
        gm.place_nuclei()
        tr = gm.run_until(X_TARGET)
        self.misses = sum(s.p_misses for s in tr)
        self.last_trace = tr
        return sum(s.Sv for s in tr), len(tr), gm.timing()

    def launches(self):
        return self.gm.timing().kernel_launches

    def timing_every(self):
        return self.gm.tune().timing_every

    def e2e(self, runs):
        sg, d, n = self.sg, self.d, self.n
        pin = [pinned_copy(x) for x in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub)]
        pd = sg.Domain(n, n, n, *pin)
        lab = pinned_copy(np.empty((n, n, n), dtype=np.uint32))
        gm = self.gm

        def once():
            gm.load_domain(pd)
            gm.place_nuclei()
            tr = gm.run_until(X_TARGET)
            gm.labels(lab)
            return sum(s.Sv for s in tr)
        once()
        t0 = time.perf_counter()
        sv = sum(once() for _ in range(runs))
        return sv, time.perf_counter() - t0, sum(x.nbytes for x in pin), lab.nbytes

    def fp32_error(self):
        """FP32+Kahan against the FP64 path (bit-exact with the reference) on the same domain."""
        lab32 = self.gm.labels()
        x32 = np.array([s.X for s in self.last_trace])
        p64 = self.sg.Params.from_buffer_copy(self.p)
        p64.precision = 0
        with self.sg.GrowthMachine(p64) as g64:
            g64.load_domain(self.d)
            g64.place_nuclei()
            tr64 = g64.run_until(X_TARGET)
            lab64 = g64.labels()
        x64 = np.array([s.X for s in tr64])
        m = min(len(x32), len(x64))
        return label_error(lab32, lab64, x32[:m], x64[:m], self.d.ndefg)

    def config(self):
        if self.pancake:
            return {"workload": f"{self.n}^3 pancake grains 1:4:8, {self.ngr} grains, 3 texture components 10 deg scatter, "
                                f"rho 1e14/5e15, {self.nnuc} grain-boundary nuclei, until X>0.99",
                    "cells": self.n ** 3, "grains": self.ngr, "nuclei": self.nnuc, "l2": "inputs larger than L2"}
        if self.recovery:
            return {"workload": f"{self.n}^3, {self.ngr} grains, {self.nnuc} nuclei with Poisson incubation times "
                                f"({NUCLEATION_RATE:g}/s), recovery rho0/(1+{RECOVERY_K} t), until X>0.99",
                    "cells": self.n ** 3, "grains": self.ngr, "nuclei": self.nnuc, "l2": "inputs larger than L2"}
        return {"workload": WORKLOAD if self.n == N_EDGE else f"{self.n}^3 at the 512^3 workload's densities",
                "cells": self.n ** 3, "grains": self.ngr, "nuclei": self.nnuc,
                "l2": "inputs larger than L2 (grid alone 512 MiB)" if self.n >= 320 else "grid smaller than L2"}

    def close(self):
        self.gm.close()


def batch_shapes(ndom: int):
    """Batched-ensemble shapes: edges uniform in [64, 256] per axis, 100-5000 grains and
    50-2000 nuclei per domain; domain i draws from seed i."""
    out = []
    for i in range(ndom):
        r = np.random.default_rng(i)
        nx, ny, nz = (int(v) for v in r.integers(64, 257, size=3))
        out.append((nx, ny, nz, int(r.integers(100, 5001)), int(r.integers(50, 2001)), i))
    return out


class BatchWorkload:
    """64 independent domains of uneven sizes stepped together (score_batch_*)."""

    def __init__(self, sg, args, rank, local):
        self.sg = sg
        self.shapes = batch_shapes(args.domains)
        self.doms, params = [], []
        with tempfile.TemporaryDirectory() as td:
            for k, (nx, ny, nz, ng, nn, seed) in enumerate(self.shapes):
                params.append(sg.read_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz, precision=args.precision).write(Path(td) / f"{k}.uds")))
                self.doms.append(sg.generate_domain(nx, ny, nz, ng, nn, seed=seed + 1000 * rank))
        self.params = params
        self.b = sg.Batch(params, device=local)
        for k, d in enumerate(self.doms):
            self.b.load_domain(k, d)
        self.tuned = self.b.autotune(X_TARGET) if args.autotune else None
        self.misses = None

    def run(self):
        b = self.b
        b.restart()
        b.place_nuclei()
        steps = b.run_until(X_TARGET)
        traces = [b.trace(k) for k in range(len(self.doms))]
        self.last_traces = traces
        self.misses = sum(s.p_misses for t in traces for s in t)
        return sum(s.Sv for t in traces for s in t), steps, b.timing()

    def launches(self):
        return self.b.timing().kernel_launches

    def timing_every(self):
        return self.b.tune().timing_every

    def e2e(self, runs):
        sg, b = self.sg, self.b
        pins, labs = [], []
        for d in self.doms:
            pin = [pinned_copy(x) for x in (d.grid, d.defg_quat, d.defg_rho0, d.rxg_quat, d.rxg_site, d.rxg_tincub)]
            pins.append(sg.Domain(d.nx, d.ny, d.nz, *pin))
            labs.append(pinned_copy(np.empty((d.nz, d.ny, d.nx), dtype=np.uint32)))

        def once():
            for k, pd in enumerate(pins):
                b.load_domain(k, pd)
            b.place_nuclei()
            b.run_until(X_TARGET)
            for k, lab in enumerate(labs):
                b.labels(k, lab)
            return sum(s.Sv for k in range(len(pins)) for s in b.trace(k))
        once()
        t0 = time.perf_counter()
        sv = sum(once() for _ in range(runs))
        h2d = sum(x.nbytes for pd in pins for x in (pd.grid, pd.defg_quat, pd.defg_rho0, pd.rxg_quat, pd.rxg_site, pd.rxg_tincub))
        return sv, time.perf_counter() - t0, h2d, sum(lab.nbytes for lab in labs)

    def fp32_error(self):
        lab32 = [self.b.labels(k) for k in range(len(self.doms))]
        self.b.close()  # the FP64 batch needs the device's argument slots
        p64 = []
        for p in self.params:
            q = self.sg.Params.from_buffer_copy(p)
            q.precision = 0
            p64.append(q)
        errs = []
        with self.sg.Batch(p64) as b64:
            for k, d in enumerate(self.doms):
                b64.load_domain(k, d)
            b64.place_nuclei()
            b64.run_until(X_TARGET)
            for k, d in enumerate(self.doms):
                x32 = np.array([s.X for s in self.last_traces[k]])
                x64 = np.array([s.X for s in b64.trace(k)])
                m = min(len(x32), len(x64))
                errs.append(label_error(lab32[k], b64.labels(k), x32[:m], x64[:m], d.ndefg))
        return {"label_mismatch": max(e["label_mismatch"] for e in errs), "max_abs_dX": max(e["max_abs_dX"] for e in errs),
                "mean_grain_size_rel_err": max(e["mean_grain_size_rel_err"] for e in errs), "aggregate": "max over domains"}

    def config(self):
        cells = sum(a * b * c for a, b, c, *_ in self.shapes)
        return {"workload": f"batched ensemble: {len(self.shapes)} domains, edges uniform in [64,256] per axis, "
                            f"100-5000 grains, 50-2000 nuclei, one launch sequence per step (CUDA graph)",
                "domains": len(self.shapes), "cells": cells, "grains": sum(s[3] for s in self.shapes),
                "nuclei": sum(s[4] for s in self.shapes), "l2": "inputs larger than L2"}

    def close(self):
        self.b.close()


def label_error(lab32, lab64, x32, x64, ndefg):
    """fraction of cells with a different final label, max |dX(t)|, relative error of the
    mean recrystallized grain size (cells per recrystallized grain)."""
    lab32, lab64 = lab32.ravel(), lab64.ravel()
    def mean_size(lab):
        rx = lab[lab >= ndefg]
        return rx.size / max(1, np.unique(rx).size)
    m64 = mean_size(lab64)
    return {"label_mismatch": float(np.mean(lab32 != lab64)), "max_abs_dX": float(np.max(np.abs(x32 - x64))) if len(x32) else 0.0,
            "mean_grain_size_rel_err": abs(mean_size(lab32) - m64) / m64 if m64 else 0.0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="plain", choices=["plain", "batch", "recovery", "pancake"],
                    help="plain: one 512^3 domain (headline); batch: ensemble of uneven domains; "
                         "recovery: 512^3 with hyperbolic recovery and Poisson nucleation; pancake: 1024^3 rolled structure")
    ap.add_argument("--edge", type=int, default=N_EDGE)
    ap.add_argument("--domains", type=int, default=64, help="batch workload: number of domains")
    ap.add_argument("--precision", type=int, default=0, help="0 FP64 (bit-exact), 1 FP32+Kahan")
    ap.add_argument("--autotune", action="store_true", help="pick the launch configuration before timing")
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
    wl = (BatchWorkload if args.workload == "batch" else PlainWorkload)(sg, args, rank, local)

    for _ in range(args.warmup):
        wl.run()
    barrier(dist)
    launches0 = wl.launches()
    tot_sv, tot_steps, run_ms, grow_bytes, grow_launches, timed_steps = 0, 0, 0.0, 0.0, 0, 0
    phase = {"grow_ms": 0.0, "fill_ms": 0.0, "claim_ms": 0.0, "commit_ms": 0.0, "host_ms": 0.0, "wait_ms": 0.0,
             "weights_ms": 0.0, "pre_ms": 0.0, "post_ms": 0.0}
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            sv, ns, tm = wl.run()
            tot_sv += sv
            tot_steps += ns
            run_ms += tm.run_ms
            grow_bytes += tm.grow_bytes
            grow_launches += tm.grow_launches
            timed_steps += tm.timed_steps
            for k in phase:
                phase[k] += getattr(tm, k)
    fill_ms = phase["fill_ms"]  # over the timed steps, like grow_bytes
    # device phases are timed with CUDA events on every k-th step only (events cost device
    # time); scaled to whole runs for the breakdown
    scale = grow_launches / timed_steps if timed_steps else 0.0
    for k in ("grow_ms", "fill_ms", "claim_ms", "commit_ms"):
        phase[k] *= scale
    launches = wl.launches() - launches0
    barrier(dist)
    t_max = reduce_max(dist, run_ms / 1e3)
    sv_all = reduce_sum(dist, float(tot_sv))
    value = sv_all / t_max

    # end to end through the C ABI: pinned host inputs in, labels out, every run
    e_value, h2d, d2h = None, 0, 0
    if not args.no_e2e:
        runs = max(1, min(args.steps, 3))
        barrier(dist)
        e_sv, e_s, h2d, d2h = wl.e2e(runs)
        barrier(dist)
        e_s = reduce_max(dist, e_s)
        e_value = reduce_sum(dist, float(e_sv)) / e_s
    every = wl.timing_every()
    fp32_err = wl.fp32_error() if args.precision == 1 else None
    wl.close()

    if rank == 0:
        peak, peak_kind = measured_peak_gbs()
        bpu = BYTES_PER_UPDATE[args.precision]
        achieved = grow_bytes / (fill_ms / 1e3) / 1e9 if fill_ms > 0 else 0.0
        traffic = None
        tf = ROOT / "profiles" / "grow_traffic.json"
        if tf.exists() and args.workload == "plain" and args.precision == 0:
            try:
                tj = json.loads(tf.read_text())
                traffic = tj["dram_bytes_per_update"] * (grow_bytes / bpu) / max(1, timed_steps)
            except Exception:
                traffic = None
        cfg = wl.config()
        cfg.update({"growth_steps_per_run": tot_steps // args.steps, "updates_per_run": tot_sv // args.steps,
                    "time_to_X099_ms": run_ms / args.steps, "parallelism": f"{world} independent ranks",
                    "phase_ms_per_run": {k: v / args.steps for k, v in phase.items()},
                    "phase_sampling": f"device phases (grow, fill, claim, commit) timed with CUDA events on {timed_steps} "
                                      f"of {grow_launches} steps (every {every}th) and scaled to the runs; "
                                      f"roofline over the timed fill launches; host phases every step",
                    "host_weight_misses_per_run": wl.misses})
        if wl.tuned is not None:
            t = wl.tuned
            cfg["autotuned"] = {"items": t.items, "fill_blocks_per_sm": t.fill_blocks_per_sm,
                                "claim_blocks_per_sm": t.claim_blocks_per_sm, "commit_blocks_per_sm": t.commit_blocks_per_sm}
        if fp32_err is not None:
            cfg["fp32_error_vs_fp64"] = fp32_err
        line = {
            "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": run_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == 0 else "f32+kahan", "data": "synthetic",
            "config": cfg,
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
