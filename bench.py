#!/usr/bin/env python
"""Benchmark: atom-timesteps/s of the 1M-atom LJ NVE step (mixed precision vs FP64).

Workload (the benchmark's configuration 1): N = 1,048,576 LJ atoms
(eps = 1, sigma = 1, cut 2.5 sigma') on a 128x128x64 simple-cubic lattice at
number density 0.8 sigma'^-3 with a +-0.05 sigma' jitter, Gaussian velocities
at T = 1, neighbour-list skin 0.3 sigma', CollectionVerlet with dt = 0.002.
A "step" is one time step of the whole system (drift, pair forces, kick,
rebuild test, and the list rebuild whenever the test fires).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun every rank runs an independent
replica of the system (the single-system step has no data-parallel split).
"""
from __future__ import annotations

import argparse
import json
import math
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

METRIC = "atom-timesteps/s (1M LJ, mixed vs FP64) at stated error"
UNIT = "atom-timesteps/s"
DT = 0.002
SHAPE = (128, 128, 64)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """Largest `value` over all ranks (the slowest replica sets the job time)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(atoms_per_rank: int, steps: int, ms_max: float, world: int) -> float:
    """Whole-job atom-timesteps/s: every rank advances its own replica (weak scaling)."""
    return world * atoms_per_rank * steps / (ms_max / 1000.0)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def traffic_from_profiles(kernel: str):
    """DRAM bytes per launch of `kernel` on this workload from its committed ncu summary."""
    p = ROOT / "profiles" / f"{kernel}_lj1m.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class Clocks:
    """Sample nvidia-smi clocks / throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_system(w, precision, device):
    from parm_gb300 import System
    s = System(w.sizes, ndim=w.ndim, precision=precision)
    s.set_boxes(w.L)
    s.set_atoms(x=w.x, v=w.v, a=np.zeros_like(w.x), f=np.zeros_like(w.x), m=w.m)
    s.set_interaction(w.kind, w.params, w.skin)
    # Collection::initialize
    s.nlist_update(False)
    s.set_forces(True)
    s.nlist_update(False)
    return s


def cpu_baseline_sample(w, max_steps=3):
    """Time the oracle (a single-threaded restatement of the reference step) on the same system.

    The reference's O(N^2) list build is infeasible at 1M atoms; the list is
    installed through the oracle's cell-list construction (same pair set, not
    timed) and only time steps without a rebuild are timed.  The O(N^2)
    rebuild cost is measured at 16384 atoms and extrapolated by N^2.
    """
    from oracle.oracle import Oracle
    o = Oracle(w.n, 3)
    o.set_box(w.L[0])
    o.set_state(x=w.x, v=w.v, a=np.zeros_like(w.x), f=np.zeros_like(w.x), m=w.m)
    o.set_interaction(w.kind, w.params, w.skin)
    o.build_fast()
    o.set_forces(True)
    which0 = o.which()
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        o.verlet(DT, 1)
        steps += 1
        if time.perf_counter() - t0 > 25:
            break
    dt = time.perf_counter() - t0
    rebuilt = o.which() != which0
    # O(N^2) rebuild at 16384 atoms
    from parm_gb300 import workloads as W
    ws = W.lj_lattice(shape=(32, 32, 16), skin_prime=0.3)
    os_ = Oracle(ws.n, 3)
    os_.set_box(ws.L[0])
    os_.set_state(x=ws.x, v=ws.v, m=ws.m)
    os_.set_interaction(ws.kind, ws.params, ws.skin)
    t1 = time.perf_counter()
    os_.nl_update(True)
    tb = time.perf_counter() - t1
    t_rebuild_1m = tb * (w.n / ws.n) ** 2
    del o, os_
    return {"value": w.n * steps / dt, "steps": steps, "seconds": dt, "rebuilt": rebuilt,
            "rebuild_s_16k": tb, "rebuild_s_extrapolated": t_rebuild_1m}


def _replica_steps(job):
    """One host thread: time `steps` oracle steps of an independent replica (spawned process)."""
    seed, steps = job
    import numpy as np_
    from oracle.oracle import Oracle
    from parm_gb300 import workloads as W
    w = W.lj_lattice(shape=SHAPE, skin_prime=0.3, seed=seed)
    o = Oracle(w.n, 3)
    o.set_box(w.L[0])
    o.set_state(x=w.x, v=w.v, a=np_.zeros_like(w.x), f=np_.zeros_like(w.x), m=w.m)
    o.set_interaction(w.kind, w.params, w.skin)
    o.build_fast()
    o.set_forces(True)
    t0 = time.perf_counter()
    o.verlet(DT, steps)
    return w.n * steps, time.perf_counter() - t0, t0


def run_reference(args, rank):
    """The reference's CPU step (the oracle port, bit-exact with it) on every host thread.

    Each host thread runs an independent replica of the 1M-atom system (the
    reference step is single-threaded); value = all replicas' atom-steps over
    the wall time from the first start to the last finish.
    """
    import multiprocessing as mp
    from oracle.build import build as build_oracle
    build_oracle()
    ncpu = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    nrep = max(1, min(ncpu, 64))
    steps = max(1, min(args.steps, 3))
    ctx = mp.get_context("spawn")
    with ctx.Pool(nrep) as pool:
        res = pool.map(_replica_steps, [(12345 + r, steps) for r in range(nrep)])
    total = sum(r[0] for r in res)
    wall = max(r[2] + r[1] for r in res) - min(r[2] for r in res)
    value = total / wall
    n = res[0][0] // steps
    sample = (f"oracle port of the reference step (bit-exact with the reference's compiled sources), "
              f"{nrep} independent {n}-atom replicas, one per host thread, {steps} CollectionVerlet steps "
              f"each without a list rebuild ({wall:.1f} s wall); the reference's O(N^2) list rebuild "
              f"(~1.8e4 s per rebuild at this size, extrapolated from 16384 atoms) is excluded")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
           "warmup": 0, "ms_per_step": 1000 * wall / steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": f"lj_nve_{n}_atoms", "n_atoms": n, "dt": DT,
                      "skin_sigma": 0.3 * 2.0 ** (-1.0 / 6.0), "lattice": list(SHAPE),
                      "replicas": nrep},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": nrep, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch
    from parm_gb300 import capi, workloads as W
    from parm_gb300.system import System
    lib = capi.load()
    capi.check(lib.parm_use_device(local_rank))
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    w = W.lj_lattice(shape=SHAPE, skin_prime=0.3, seed=12345 + rank)
    n = w.n
    log(f"[rank {rank}] building mixed system, n={n}")
    g = make_system(w, "mixed", local_rank)
    g.set_graph_steps(args.graph_steps)
    tpa = g.autotune() if args.tpa == 0 else (g.set_threads_per_atom(args.tpa) or args.tpa)
    log(f"[rank {rank}] threads per atom: {tpa}")
    g.verlet(DT, args.warmup)
    g.sync()
    e_start = g.energy()[0] + g.kinetic_energy()[0]
    stream = torch.cuda.ExternalStream(g.stream())
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local_rank)
    g.timing(True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(stream)
    g.verlet(DT, args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = g.last_launches()
    tr = g.timing_read()
    g.timing(False)
    if dist:
        ms = max_over_ranks(ms, dist, "cuda")
        dist.barrier()
    e_end = g.energy()[0] + g.kinetic_energy()[0]
    value = job_throughput(n, args.steps, ms, world)
    npairs = int(g.numpairs()[0])

    # --- roofline of the dominant kernel (the mixed pair-force kernel) ---
    # algorithmic bytes per atom and launch: the atom's FP32 position record
    # (32 B, each read once), its pair parameters (16 B) and list length (4 B),
    # its list entries (2 B each for the cell-block kernel, 4 B for the
    # gather kernel) and its force (16 B written)
    force_ms = tr["force_ms"] / max(1, tr["force_launches"])
    nnb = 2.0 * npairs / n   # full-list entries per atom
    staged = tpa == 2000 or tpa == 200
    kernel = "k_force_stg" if staged else "k_force32"
    bytes_per_atom = 32.0 + 16.0 + 4.0 + 16.0 + (2.0 if staged else 4.0) * nnb
    algo_bytes = n * bytes_per_atom
    achieved = algo_bytes / (force_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = traffic_from_profiles(kernel)

    result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (mixed)", "data": "synthetic",
              "config": {"workload": f"lj_nve_{n}_atoms_mixed", "n_atoms": n, "lattice": list(SHAPE),
                         "box": [float(v) for v in w.L[0]], "dt": DT, "skin_sigma": w.skin,
                         "cutoff_sigma": float(w.params[0, 2]), "precision": "mixed",
                         "parallelism": f"replicas{world}" if world > 1 else "single",
                         "l2": "inputs larger than L2 (state + neighbour lists ~1 GB)",
                         "steps_per_graph": args.graph_steps, "threads_per_atom": tpa},
              "clocks": ck,
              "gpu_launches": launches,
              "rebuilds": tr["rebuilds"]}
    result["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": traffic,
                          "kernel": f"{kernel} (mixed-precision pair forces)",
                          "algorithmic_bytes_per_atom": bytes_per_atom,
                          "algorithmic_bytes_per_launch": algo_bytes, "force_ms_per_launch": force_ms,
                          "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                          else "fallback 6800 GB/s"}
    result["energy_drift_rel"] = {"per_1e5_steps": abs(e_end - e_start) / abs(e_start) * 1e5 / args.steps,
                                  "steps": args.steps}

    if args.only_timed:
        g.close()
        if rank == 0:
            print(json.dumps(result), flush=True)
        return

    # --- FP64 path on the same system, and mixed-vs-FP64 error at one state ---
    st = g.get_atoms(capi.X | capi.V | capi.A)
    w64 = W.lj_lattice(shape=SHAPE, skin_prime=0.3, seed=12345 + rank)
    w64.x, w64.v = st["x"], st["v"]
    g64 = make_system(w64, "fp64", local_rank)
    g64.set_graph_steps(10)
    k64 = max(3, min(40, args.steps // 10))
    g64.verlet(DT, 2)
    torch.cuda.synchronize()
    s64 = torch.cuda.ExternalStream(g64.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s64)
    g64.verlet(DT, k64)
    e1.record(s64)
    e1.synchronize()
    v64 = n * k64 / (e0.elapsed_time(e1) / 1000.0)
    # forces at one common state
    st64 = g64.get_atoms(capi.X)
    g.set_atoms(x=st64["x"])
    g.nlist_update(True)
    g64.nlist_update(True)
    g.set_forces(False)
    g64.set_forces(False)
    F32 = g.get_atoms(capi.F)["f"]
    F64 = g64.get_atoms(capi.F)["f"]
    ferr = float(np.sqrt(((F32 - F64) ** 2).sum(1)).max() / np.sqrt((F64 ** 2).sum(1).mean()))
    E32, E64 = g.energy()[0], g64.energy()[0]
    result["fp64_value"] = world * v64
    result["mixed_vs_fp64"] = value / (world * v64)
    result["accuracy"] = {"max_force_err_over_rms_force": ferr, "rel_energy_err": abs(E32 - E64) / abs(E64)}
    g64.close()

    # --- end to end through the C ABI with host buffers ---
    stride = 4 * 3 + 1
    nbytes = n * stride * 8
    import ctypes as C
    hp = C.c_void_p()
    capi.check(lib.parm_host_alloc(C.byref(hp), nbytes))
    buf = np.ctypeslib.as_array((C.c_double * (n * stride)).from_address(hp.value)).reshape(n, stride)
    cur = g.get_atoms()
    buf[:, 0:3], buf[:, 3:6], buf[:, 6:9], buf[:, 9:12], buf[:, 12] = cur["x"], cur["v"], cur["a"], cur["f"], cur["m"]
    fields = capi.X | capi.V | capi.A | capi.F | capi.M   # whole Atom records, as an AtomVec holds them
    dptr = buf.ctypes.data_as(C.POINTER(C.c_double))
    n_e2e = max(3, min(args.e2e_steps, args.steps))
    for _ in range(2):
        capi.check(lib.parm_set_atoms(g.h, dptr, stride, fields))
        capi.check(lib.parm_verlet(g.h, DT, 1))
        capi.check(lib.parm_get_atoms(g.h, dptr, stride, fields))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        capi.check(lib.parm_set_atoms(g.h, dptr, stride, fields))
        capi.check(lib.parm_verlet(g.h, DT, 1))
        capi.check(lib.parm_get_atoms(g.h, dptr, stride, fields))
    t_e2e = time.perf_counter() - t0
    if dist:
        t_e2e = max_over_ranks(t_e2e, dist, "cuda")
    result["e2e"] = {"value": world * n * n_e2e / t_e2e, "unit": UNIT, "h2d_bytes_per_step": n * stride * 8,
                     "d2h_bytes_per_step": n * stride * 8, "steps": n_e2e,
                     "api": "parm_set_atoms + parm_verlet(dt, 1) + parm_get_atoms on whole Atom records "
                            "{x,v,a,f,m} in pinned host memory"}
    lib.parm_host_free(hp)
    g.close()

    if rank == 0 and world == 1 and not args.no_cpu:
        log("[rank 0] timing the CPU oracle sample")
        s = cpu_baseline_sample(w)
        result["cpu_baseline"] = {
            "value": s["value"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": (f"oracle port, {s['steps']} CollectionVerlet steps of the same {n}-atom system on one "
                       f"host thread ({s['seconds']:.1f} s), list installed by the cell-list construction "
                       f"(untimed); reference O(N^2) rebuild: {s['rebuild_s_16k']:.2f} s at 16384 atoms, "
                       f"~{s['rebuild_s_extrapolated']:.0f} s extrapolated to {n} (excluded)")}
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--graph-steps", type=int, default=50,
                    help="time steps per CUDA graph launch (0: direct kernel launches, for profilers)")
    ap.add_argument("--tpa", type=int, default=0,
                    help="pair-kernel variant (0: autotune; 1/2/4 tiled, 100+t gather)")
    ap.add_argument("--only-timed", action="store_true",
                    help="run only the timed mixed-precision region (used for profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args, rank)
        return
    run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
