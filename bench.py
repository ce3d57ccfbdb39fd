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
SCORE reference's sources are not on the GPU host) on the same 512^3 workload, one
whole run per process on every host core, like the reference's MPI ensemble of
solitary units; loop time only; rank 0 only.
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


REF_RSS_BYTES = 3.0e9     # peak resident memory of one 512^3 oracle process (2.4 GB measured) with headroom
REF_WARM_EDGE = 64        # warm-up domains of the reference arm: same densities, 64^3


def _mem_available() -> float:
    try:
        for line in Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                return float(line.split()[1]) * 1024.0
    except OSError:
        pass
    return 0.0


def _ref_worker(conn, shared: str):
    """One process of the reference arm: the headline workload's 512^3 domain (shared by
    the parent as .npy files in `shared`, mapped read-only), stepped by the oracle port in
    pieces on command.  Nothing here loads the CUDA library."""
    sys.path.insert(0, str(ROOT))
    import score_gb300 as sg
    import oracle
    try:
        def load(tag):
            a = [np.load(Path(shared) / f"{tag}_{k}.npy", mmap_mode="r") for k in range(6)]
            return sg.Domain(int(a[0].shape[2]), int(a[0].shape[1]), int(a[0].shape[0]), *a)
        d, dw = load("main"), load("warm")
        p, pw = read_params(N_EDGE), read_params(REF_WARM_EDGE)
        sim = oracle.Sim(p, d)
        conn.send(("ready", None))
        while True:
            cmd, arg = conn.recv()
            if cmd == "warm":      # one whole same-density 64^3 run (untimed)
                oracle.run(pw, dw, x_target=X_TARGET)
                conn.send(("ok", None))
            elif cmd == "advance":  # the 512^3 run up to X > arg: this piece's updates, steps and loop seconds
                r = sim.advance(x_target=arg)
                conn.send(("ok", (int(r["trace"]["Sv"].sum()), int(r["n_steps"]), float(r["seconds"]), int(r["status"]))))
            else:
                sim.close()
                conn.send(("ok", None))
                return
    except Exception as e:  # reported to the parent, which stops the arm
        conn.send(("error", repr(e)))


def run_reference_arm(args) -> None:
    """The reference's CPU algorithm (the C oracle port of solve_RXGROWTH) on the host cores,
    on the headline workload itself: every process steps the GPU arm's 512^3 domain (20,000
    grains, 50,000 nuclei, seed 0, the same physics) from nucleation to X > 0.99, like the
    reference's ensemble of solitary units over MPI ranks.  The parent makes the inputs
    once, before the timed region, and shares them through files in /dev/shm.  Bench step k advances every process's run to
    X > 0.99 k / steps; its time is the longest process's loop time of that piece, so the
    timed steps cover exactly one whole run per process.  Warm-up steps run whole
    same-density 64^3 domains.  Under torchrun only rank 0 works and prints."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    import oracle
    import score_gb300 as sg
    sg.build()          # host-only library for the inputs (the CUDA library is not loaded)
    oracle.build_oracle()
    cores = os.cpu_count() or 1
    avail = _mem_available()
    # one oracle process per core, as many as the host's free memory holds (the shared inputs aside)
    nproc = max(1, min(cores, int(0.8 * (avail - 1.5e9) / REF_RSS_BYTES))) if avail > 0 else cores
    t_setup = time.perf_counter()
    shm = Path("/dev/shm") if Path("/dev/shm").is_dir() else Path(tempfile.gettempdir())
    shared = Path(tempfile.mkdtemp(prefix="score_refarm_", dir=shm))
    fw = (REF_WARM_EDGE / N_EDGE) ** 3
    for tag, dom in (("main", sg.generate_domain(N_EDGE, N_EDGE, N_EDGE, N_GRAINS, N_NUCLEI, seed=0)),
                     ("warm", sg.generate_domain(REF_WARM_EDGE, REF_WARM_EDGE, REF_WARM_EDGE, max(1, round(N_GRAINS * fw)),
                                                 max(1, round(N_NUCLEI * fw)), seed=1))):
        for k, a in enumerate((dom.grid, dom.defg_quat, dom.defg_rho0, dom.rxg_quat, dom.rxg_site, dom.rxg_tincub)):
            np.save(shared / f"{tag}_{k}.npy", a)
        del dom
    ctx = mp.get_context("spawn")
    pipes, procs = [], []
    for i in range(nproc):
        a, b = ctx.Pipe()
        pr = ctx.Process(target=_ref_worker, args=(b, str(shared)), daemon=True)
        pr.start()
        pipes.append(a)
        procs.append(pr)

    def gather():
        out = []
        for c in pipes:
            tag, val = c.recv()
            if tag == "error":
                raise RuntimeError(f"reference arm worker failed: {val}")
            out.append(val)
        return out

    try:
        gather()  # every process has its inputs
        t_setup = time.perf_counter() - t_setup
        for _ in range(args.warmup):
            for c in pipes:
                c.send(("warm", None))
            gather()
        tot_sv, tot_s, tot_steps = 0, 0.0, 0
        for k in range(1, args.steps + 1):
            xt = X_TARGET * k / args.steps
            for c in pipes:
                c.send(("advance", xt))
            res = gather()
            if any(r[3] != 0 for r in res):
                raise RuntimeError(f"oracle status {[r[3] for r in res]}")
            tot_sv += sum(r[0] for r in res)
            tot_steps += max(r[1] for r in res)
            tot_s += max(r[2] for r in res)
        for c in pipes:
            c.send(("close", None))
        gather()
    finally:
        for pr in procs:
            pr.join(timeout=30)
            if pr.is_alive():
                pr.kill()
        import shutil
        shutil.rmtree(shared, ignore_errors=True)
    v = tot_sv / tot_s
    sample = (f"C oracle port of solve_RXGROWTH (the reference's sources are not on this host), {nproc} processes on "
              f"{cores} host cores, each one whole run of the 512^3 workload's domain (seed 0) from nucleation to X>0.99, "
              f"split into {args.steps} pieces by X; loop time only (inputs made before, {t_setup:.0f} s)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "updates/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": N_EDGE ** 3, "grains": N_GRAINS, "nuclei": N_NUCLEI,
                       "processes": nproc, "runs_timed": nproc, "updates_timed": tot_sv,
                       "growth_steps_per_run": tot_steps, "mem_available_gb": round(avail / 1e9, 1)},
            "cpu_baseline": {"value": v, "unit": "updates/s", "cores": nproc, "kind": "port", "sample": sample},
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


LOGPOINTS = ["0.0", "0.1", "0.2", "0.3", "0.4", "0.5", "0.6", "0.7", "0.8", "0.9"]


def measure_synthesis(sg, local) -> dict:
    """Deformed-structure synthesis of the headline domain (512^3, 20,000 Voronoi grains, 50,000 nuclei):
    the device label fill (score_generate_domain_gpu) against the host generator on every host core,
    each the whole public call (seeds, fill, orientations, nuclei, grid in a host buffer)."""
    t0 = time.perf_counter()
    dh = sg.generate_domain(N_EDGE, N_EDGE, N_EDGE, N_GRAINS, N_NUCLEI, seed=0)
    host_s = time.perf_counter() - t0
    sg.generate_domain(64, 64, 64, 100, 10, seed=1, device=local)  # warm-up: module load
    t0 = time.perf_counter()
    dd = sg.generate_domain(N_EDGE, N_EDGE, N_EDGE, N_GRAINS, N_NUCLEI, seed=0, device=local)
    gpu_s = time.perf_counter() - t0
    same = all(np.array_equal(getattr(dh, f), getattr(dd, f)) for f in ("grid", "defg_quat", "defg_rho0", "rxg_quat", "rxg_site"))
    return {"workload": "512^3 periodic Voronoi, 20000 grains, 50000 nuclei (the headline domain)",
            "gpu_s": gpu_s, "host_s": host_s, "host_threads": os.cpu_count(), "gpu_cells_per_s": N_EDGE ** 3 / gpu_s,
            "identical": bool(same)}


def measure_postprocessing(sg, local, doms, shapes, runs: int) -> dict:
    """On-the-fly characterization and ensemble post-processing on the batched ensemble: the run with
    the grain-evolution log at 10 logpoints (counts and RX area profile, threshold 13) against the
    same run without it, then the device post-processing of the 64 logs (1000 rediscretized times:
    kinetics, and macrotexture over 8 orientation classes), timed through the public API."""
    out = {}
    with tempfile.TemporaryDirectory() as td:
        plog = [sg.read_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz, logpoints=LOGPOINTS).write(Path(td) / f"{k}.uds"))
                for k, (nx, ny, nz, *_r) in enumerate(shapes)]
    with sg.Batch(plog, device=local) as b:
        for k, d in enumerate(doms):
            b.load_domain(k, d)
        ms = 0.0
        for r in range(1 + runs):
            b.restart()
            b.place_nuclei()
            b.run_until(X_TARGET)
            if r:
                ms += b.timing().run_ms
        nsnap = sum(len(b.grainevo(k)) for k in range(len(doms)))
        grains = sum(d.ndefg + d.nrxg for d in doms)
        cls = np.concatenate([np.arange(d.ndefg + d.nrxg, dtype=np.uint32) % 8 for d in doms])
        tk, tt = [], []
        for _ in range(5):
            t0 = time.perf_counter()
            b.rediscr_kinetics(1000)
            tk.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            b.rediscr_texture(1000, cls, 8)
            tt.append(time.perf_counter() - t0)
    kin, tex = statistics.median(tk), statistics.median(tt)
    out.update({"logged_run_ms": ms / runs, "snapshots": nsnap,
                "rediscr_kinetics_ms": 1e3 * kin, "rediscr_texture_ms": 1e3 * tex,
                "interpolations_per_s_kinetics": 1000 * sum(d.ndefg for d in doms) / kin,
                "interpolations_per_s_texture": 1000 * grains / tex,
                "how": "host wall time of the public call (upload of the logs' times and classes, two kernels, download)"})
    return out


def measure_batched(sg, args, local) -> dict:
    """The metric's ratio on the batched ensemble (64 domains, edges uniform in [64, 256]
    per axis, 100-5000 grains, 50-2000 nuclei; domain i from seed i): the batched path in
    FP64 and in FP32+Kahan (updates/s over whole runs to X > 0.99, inputs resident, CUDA
    events), against the same 64 domains stepped one after another, each through its own
    single-domain context (score_run_until, FP64): the reference steps its solitary units
    one after another the same way.  FP32 error against the FP64 batch (bit-exact)."""
    shapes = batch_shapes(64)
    doms, p64, p32 = [], [], []
    with tempfile.TemporaryDirectory() as td:
        for k, (nx, ny, nz, ng, nn, seed) in enumerate(shapes):
            p64.append(sg.read_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz, precision=0).write(Path(td) / f"{k}a.uds")))
            p32.append(sg.read_uds(sg.UdsSpec(nx=nx, ny=ny, nz=nz, precision=1).write(Path(td) / f"{k}b.uds")))
            doms.append(sg.generate_domain(nx, ny, nz, ng, nn, seed=seed))
    runs = max(1, min(args.steps, 5))
    out = {"workload": "64 domains, edges uniform in [64,256] per axis, 100-5000 grains, 50-2000 nuclei, until X>0.99",
           "cells": int(sum(a * b * c for a, b, c, *_ in shapes)), "runs_timed": runs}

    def batch_rate(params):
        with sg.Batch(params, device=local) as b:
            for k, d in enumerate(doms):
                b.load_domain(k, d)
            sv, ms = 0, 0.0
            for r in range(1 + runs):  # the first run is a warm-up
                b.restart()
                b.place_nuclei()
                b.run_until(X_TARGET)
                if r:
                    sv += sum(s.Sv for k in range(len(doms)) for s in b.trace(k))
                    ms += b.timing().run_ms
            labs = [b.labels(k) for k in range(len(doms))]
            xs = [np.array([s.X for s in b.trace(k)]) for k in range(len(doms))]
            launches = b.timing().kernel_launches
        return sv / (ms / 1e3), labs, xs, ms / runs

    v64, lab64, x64, ms64 = batch_rate(p64)
    v32, lab32, x32, _ = batch_rate(p32)
    errs = []
    for k, d in enumerate(doms):
        m = min(len(x32[k]), len(x64[k]))
        errs.append(label_error(lab32[k], lab64[k], x32[k][:m], x64[k][:m], d.ndefg))
    # the same domains one after another through single-domain contexts
    gms = []
    try:
        for k, d in enumerate(doms):
            gm = sg.GrowthMachine(p64[k], device=local)
            gms.append(gm)
            gm.load_domain(d)
        sv, ms = 0, 0.0
        for r in range(1 + runs):
            for gm in gms:
                gm.restart()
                gm.place_nuclei()
                tr = gm.run_until(X_TARGET)
                if r:
                    sv += sum(s.Sv for s in tr)
                    ms += gm.timing().run_ms
        vseq = sv / (ms / 1e3)
    finally:
        for gm in gms:
            gm.close()
    post = measure_postprocessing(sg, local, doms, shapes, runs)
    post["unlogged_run_ms"] = ms64
    out["characterization"] = post
    out.update({
        "fp64_batched_updates_per_s": v64, "fp32_kahan_batched_updates_per_s": v32,
        "plain_fp64_same_domains_updates_per_s": vseq,
        "ratio_fp32_batched_vs_plain_fp64_same_domains": v32 / vseq,
        "ratio_fp64_batched_vs_plain_fp64_same_domains": v64 / vseq,
        "fp32_error_vs_fp64": {"label_mismatch": max(e["label_mismatch"] for e in errs),
                               "max_abs_dX": max(e["max_abs_dX"] for e in errs),
                               "mean_grain_size_rel_err": max(e["mean_grain_size_rel_err"] for e in errs),
                               "aggregate": "max over the 64 domains"},
        "plain_path": "each domain through score_create / score_load_domain / score_run_until, one after another"})
    return out


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
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-ensemble ratio (profiling captures)")
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
    batched = None
    if args.workload == "plain" and args.edge == N_EDGE and args.precision == 0 and not args.no_batched:
        batched = measure_batched(sg, args, local)
        batched["ratio_fp32_batched_vs_plain_fp64_512"] = batched["fp32_kahan_batched_updates_per_s"] / value
        batched["synthesis"] = measure_synthesis(sg, local)

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
        cfg["ms_per_growth_step"] = run_ms / max(1, tot_steps)
        line = {
            "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": run_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == 0 else "f32+kahan", "data": "synthetic",
            "config": cfg,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if peak else None, "traffic": traffic,
                         "kernel": "k_grow_fill (k_grow_fill_pf in grow mode 3)", "bytes_per_update": bpu, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
            "e2e": {"value": e_value, "unit": "updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        if batched is not None:
            line["batched"] = batched
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
